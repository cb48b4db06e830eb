// Flux statistics of optical depths still resident in HBM: the mean-flux
// rescaling (fake_spectra/py_module.cpp:235-282, get_mean_flux_scale /
// Py_mean_flux), the flux PDF (fake_spectra/fluxstatistics.py:42-51) and the
// 1-D flux power spectrum (fluxstatistics.py:53-110).
//
// All three read tau once per pass and are HBM-bound reductions.  Sums are
// deterministic: every block reduces a fixed contiguous range in a fixed
// order and a second pass adds the block partials in order, so a result does
// not depend on scheduling.
#include <cufft.h>

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

// Per block: sum of exp(-scale tau), sum of tau exp(-scale tau) and the count
// over the pixels with tau <= thresh (py_module.cpp:242-251).
__global__ void __launch_bounds__(RED_THREADS) flux_moments_kernel(const double *tau, long long n,
                                                                   double scale, double thresh,
                                                                   double *part)
{
    __shared__ double scratch[RED_THREADS / 32];
    long long lo, hi;
    block_range(n, lo, hi);
    double f = 0.0, tf = 0.0, cnt = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += RED_THREADS) {
        const double t = tau[i];
        if (t > thresh)
            continue;
        const double e = exp(-scale * t);
        f += e;
        tf += e * t;
        cnt += 1.0;
    }
    f = block_sum_ordered(f, scratch);
    tf = block_sum_ordered(tf, scratch);
    cnt = block_sum_ordered(cnt, scratch);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = f;
        part[3 * blockIdx.x + 1] = tf;
        part[3 * blockIdx.x + 2] = cnt;
    }
}

// Sum of exp(-scale tau) over all pixels (np.mean(np.exp(-tau)) with scale 1).
__global__ void __launch_bounds__(RED_THREADS) flux_sum_kernel(const double *tau, long long n,
                                                               double scale, double *part)
{
    __shared__ double scratch[RED_THREADS / 32];
    long long lo, hi;
    block_range(n, lo, hi);
    double f = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += RED_THREADS)
        f += exp(-scale * tau[i]);
    f = block_sum_ordered(f, scratch);
    if (threadIdx.x == 0)
        part[blockIdx.x] = f;
}

// In-order sum of `width`-strided block partials (one thread per component).
__global__ void partial_sum_kernel(const double *part, int nblocks, int width, double *out)
{
    const int c = threadIdx.x;
    if (c >= width)
        return;
    double t = 0.0;
    for (int b = 0; b < nblocks; b++)
        t += part[(size_t)b * width + c];
    out[c] = t;
}

// np.histogram with explicit edges (numpy's sorted-search rule): bin j holds
// e_j <= x < e_{j+1}, the last bin also x == e_last; values outside
// [e_0, e_last] and NaN are not counted.  x = exp(-scale tau).
__global__ void flux_hist_kernel(const double *tau, long long n, double scale, const double *edges,
                                 int nb, unsigned long long *counts)
{
    extern __shared__ unsigned long long hist[];
    for (int j = threadIdx.x; j < nb; j += blockDim.x)
        hist[j] = 0ull;
    __syncthreads();
    const double e0 = edges[0], el = edges[nb];
    const double norm = nb / (el - e0);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double x = exp(-scale * tau[i]);
        if (!(x >= e0 && x <= el))
            continue;
        int j = (int)((x - e0) * norm);
        j = j < 0 ? 0 : (j > nb - 1 ? nb - 1 : j);
        while (j > 0 && x < edges[j])
            j--;
        while (j < nb - 1 && x >= edges[j + 1])
            j++;
        atomicAdd(&hist[j], 1ull);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nb; j += blockDim.x)
        if (hist[j])
            atomicAdd(&counts[j], hist[j]);
}

// dflux = exp(-scale tau) / mean_flux - 1 for `rows` sightlines.
__global__ void dflux_kernel(const double *tau, long long count, double scale, double inv_mean,
                             double *out)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
        out[i] = exp(-scale * tau[i]) * inv_mean - 1.0;
}

// power[k] += vmax * sum_rows |F_row(k)|^2 / npix^2, rows in order (one thread per k).
__global__ void power_accumulate_kernel(const cufftDoubleComplex *F, int rows, int nk, int npix,
                                        double vmax, double *power)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk)
        return;
    const double inv = 1.0 / ((double)npix * (double)npix);
    double t = 0.0;
    for (int r = 0; r < rows; r++) {
        const cufftDoubleComplex z = F[(size_t)r * nk + k];
        t += (z.x * z.x + z.y * z.y) * inv;
    }
    power[k] += vmax * t;
}

}  // namespace

void launch_flux_moments(const double *tau, long long n, double scale, double thresh,
                         double *part, double *out3, cudaStream_t s)
{
    flux_moments_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(tau, n, scale, thresh, part);
    partial_sum_kernel<<<1, 32, 0, s>>>(part, RED_BLOCKS, 3, out3);
}

void launch_flux_sum(const double *tau, long long n, double scale, double *part, double *out1,
                     cudaStream_t s)
{
    flux_sum_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(tau, n, scale, part);
    partial_sum_kernel<<<1, 32, 0, s>>>(part, RED_BLOCKS, 1, out1);
}

size_t flux_partials(int width) { return (size_t)RED_BLOCKS * width; }

void launch_flux_hist(const double *tau, long long n, double scale, const double *edges, int nb,
                      unsigned long long *counts, cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = sizeof(unsigned long long) * nb;
    cudaFuncSetAttribute(flux_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    flux_hist_kernel<<<sms * 4, 256, smem, s>>>(tau, n, scale, edges, nb, counts);
}

void launch_dflux(const double *tau, long long count, double scale, double inv_mean, double *out,
                  cudaStream_t s)
{
    const long long blocks = (count + 255) / 256;
    dflux_kernel<<<(unsigned)(blocks < 65535 ? (blocks > 0 ? blocks : 1) : 65535), 256, 0, s>>>(
        tau, count, scale, inv_mean, out);
}

void launch_power_accumulate(const void *F, int rows, int nk, int npix, double vmax,
                             double *power, cudaStream_t s)
{
    power_accumulate_kernel<<<(nk + 127) / 128, 128, 0, s>>>(
        (const cufftDoubleComplex *)F, rows, nk, npix, vmax, power);
}

}  // namespace fsg
