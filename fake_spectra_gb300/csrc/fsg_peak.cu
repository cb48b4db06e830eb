// FMA-pipe peak microbenchmark (FP32 and FP64), used as the roofline
// denominator of the compute-bound deposit kernel.  Each thread runs eight
// independent dependent chains x = fma(x, a, b); 2 flops per FMA.
#include "fsg_internal.cuh"

namespace fsg {

namespace {

template <class T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T *out, int iters, T a, T b)
{
    T x0 = (T)threadIdx.x * (T)1e-6, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
    T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            x0 = fma(x0, a, b);
            x1 = fma(x1, a, b);
            x2 = fma(x2, a, b);
            x3 = fma(x3, a, b);
            x4 = fma(x4, a, b);
            x5 = fma(x5, a, b);
            x6 = fma(x6, a, b);
            x7 = fma(x7, a, b);
        }
    }
    const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == (T)-12345.678)   // never true; keeps the chains alive
        out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class T>
double run(int iters, cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256;
    T *out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess)
        return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const T a = (T)0.999999, b = (T)1e-7;
    fma_chain_kernel<T><<<blocks, threads, 0, s>>>(out, iters / 8, a, b);   // warm-up
    double best = 0.0;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(e0, s);
        fma_chain_kernel<T><<<blocks, threads, 0, s>>>(out, iters, a, b);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
        const double tf = flops / (ms * 1e-3) / 1e12;
        if (tf > best)
            best = tf;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return best;
}

}  // namespace

double measure_fma_peak(int precision, cudaStream_t s)
{
    return precision == 0 ? run<double>(64, s) : run<float>(4096, s);
}

}  // namespace fsg
