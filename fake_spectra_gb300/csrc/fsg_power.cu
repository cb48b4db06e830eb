// 1-D flux power spectrum (fake_spectra/fluxstatistics.py:53-110) with the
// project's own FP64 discrete Fourier transforms.
//
// The reference takes np.fft.rfft of d_F = exp(-s tau) / <F> - 1 along each
// sightline and sums |rfft|^2 / npix^2 over sightlines.  Here two sightlines a
// and b go through one complex transform of z = d_a + i d_b: with Z the
// transform of z, A and B those of d_a and d_b,
//     A_k = (Z_k + conj Z_{N-k}) / 2,   B_k = (Z_k - conj Z_{N-k}) / (2i),
// and by the parallelogram law |A_k|^2 + |B_k|^2 = (|Z_k|^2 + |Z_{N-k}|^2) / 2,
// so the pair's power needs no separation step and the work per sightline is
// half a complex transform, for every length N.
//
// Transforms: the self-sorting Stockham form of the mixed-radix Cooley-Tukey
// algorithm (one pass per radix, as formulated for GPUs by Govindaraju et al.,
// "High performance discrete Fourier transforms on graphics processors", SC
// 2008), radices 16/8/4/2 in registers and odd radices up to 63 by the direct
// DFT with the symmetric pairing of j and R - j (cos and sin sums over half the
// terms).  A length with a prime factor above 63 uses Bluestein's chirp-z
// algorithm over a 7-smooth length M >= 2N - 1: X_k = w_k (a * b)_k with
// w_n = exp(-i pi n^2 / N), a_n = z_n w_n, b_n = conj w_n, the circular
// convolution as conj(FFT(conj(FFT(a) FFT(b)))) / M; |w_k| = 1, so the power is
// |FFT(conj(FFT(a) FFT(b)))_k|^2 / M^2.
//
// GB300 runs FP64 at 1/64 of the FP32 rate, and the transform is FP64-bound
// (the reference's test tolerance of 1e-10 relative leaves no room for FP32
// arithmetic): the passes keep every table (twiddles, cos/sin of the odd
// radices) precomputed, and the odd-radix DFT costs about R FMAs per point.
// Memory traffic (one read and one write of 16 bytes per point and pass) is
// secondary.  Sums over sightlines go in a fixed order: fixed segments of
// pairs, each summed in order, then the segments in order.
#include "fsg_fexp.cuh"
#include "fsg_internal.cuh"

namespace fsg {

namespace {

constexpr int PASS_THREADS = 256;
constexpr int POWER_SEGMENTS = 64;   // fixed: the summation order does not depend on the GPU

__device__ __forceinline__ double2 cadd(double2 a, double2 b)
{
    return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ double2 csub(double2 a, double2 b)
{
    return make_double2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// -i a
__device__ __forceinline__ double2 mul_mi(double2 a) { return make_double2(a.y, -a.x); }

// exp(-i pi E / 8) a, E in 0..15 known at compile time.
template <int E>
__device__ __forceinline__ double2 rot16(double2 a)
{
    constexpr double H = 0.70710678118654752440;    // cos(pi/4)
    constexpr double C1 = 0.92387953251128675613;   // cos(pi/8)
    constexpr double S1 = 0.38268343236508977173;   // sin(pi/8)
    if constexpr (E == 0)
        return a;
    else if constexpr (E == 4)
        return mul_mi(a);
    else if constexpr (E == 8)
        return make_double2(-a.x, -a.y);
    else if constexpr (E == 2)
        return make_double2(H * (a.x + a.y), H * (a.y - a.x));
    else if constexpr (E == 6)
        return make_double2(H * (a.y - a.x), -H * (a.x + a.y));
    else if constexpr (E == 1)
        return cmul(a, make_double2(C1, -S1));
    else if constexpr (E == 3)
        return cmul(a, make_double2(S1, -C1));
    else if constexpr (E == 9)
        return cmul(a, make_double2(-C1, S1));
    else
        static_assert(E == 0, "rotation not used by the 8- and 16-point DFTs");
}

__device__ __forceinline__ void dft2(double2 &a, double2 &b)
{
    const double2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

// In-place forward DFT of 4 points, natural order.
__device__ __forceinline__ void dft4(double2 &x0, double2 &x1, double2 &x2, double2 &x3)
{
    const double2 t0 = cadd(x0, x2), t1 = csub(x0, x2);
    const double2 t2 = cadd(x1, x3), t3 = mul_mi(csub(x1, x3));
    x0 = cadd(t0, t2);
    x2 = csub(t0, t2);
    x1 = cadd(t1, t3);
    x3 = csub(t1, t3);
}

// Forward DFT of R points held in registers, natural order in and out.  R = 8
// and 16 split as R1 x R2 (R1 = 4): n = R2 n1 + n2, k = k1 + R1 k2: R2 DFTs of 4
// on the stride-R2 subsequences, the twiddles exp(-2 pi i n2 k1 / R), then 4
// DFTs of R2 across them.
template <int R>
__device__ __forceinline__ void dft(double2 (&v)[R]);

template <>
__device__ __forceinline__ void dft<2>(double2 (&v)[2])
{
    dft2(v[0], v[1]);
}

template <>
__device__ __forceinline__ void dft<4>(double2 (&v)[4])
{
    dft4(v[0], v[1], v[2], v[3]);
}

template <int K1, int N2, int R>
__device__ __forceinline__ double2 twid(double2 a)
{
    return rot16<(16 / R) * N2 * K1>(a);
}

template <>
__device__ __forceinline__ void dft<8>(double2 (&v)[8])
{
    // n = 2 n1 + n2
    dft4(v[0], v[2], v[4], v[6]);
    dft4(v[1], v[3], v[5], v[7]);
    // y[n2][k1] sits at v[2 k1 + n2]
    v[3] = twid<1, 1, 8>(v[3]);
    v[5] = twid<2, 1, 8>(v[5]);
    v[7] = twid<3, 1, 8>(v[7]);
    double2 o[8];
    o[0] = cadd(v[0], v[1]);
    o[4] = csub(v[0], v[1]);
    o[1] = cadd(v[2], v[3]);
    o[5] = csub(v[2], v[3]);
    o[2] = cadd(v[4], v[5]);
    o[6] = csub(v[4], v[5]);
    o[3] = cadd(v[6], v[7]);
    o[7] = csub(v[6], v[7]);
#pragma unroll
    for (int i = 0; i < 8; i++)
        v[i] = o[i];
}

template <>
__device__ __forceinline__ void dft<16>(double2 (&v)[16])
{
    // n = 4 n1 + n2: after the first DFTs y[n2][k1] sits at v[4 k1 + n2]
    dft4(v[0], v[4], v[8], v[12]);
    dft4(v[1], v[5], v[9], v[13]);
    dft4(v[2], v[6], v[10], v[14]);
    dft4(v[3], v[7], v[11], v[15]);
    v[5] = twid<1, 1, 16>(v[5]);
    v[9] = twid<2, 1, 16>(v[9]);
    v[13] = twid<3, 1, 16>(v[13]);
    v[6] = twid<1, 2, 16>(v[6]);
    v[10] = twid<2, 2, 16>(v[10]);
    v[14] = twid<3, 2, 16>(v[14]);
    v[7] = twid<1, 3, 16>(v[7]);
    v[11] = twid<2, 3, 16>(v[11]);
    v[15] = twid<3, 3, 16>(v[15]);
    // X[k1 + 4 k2] = DFT4 over n2 of y[n2][k1]
    dft4(v[0], v[1], v[2], v[3]);
    dft4(v[4], v[5], v[6], v[7]);
    dft4(v[8], v[9], v[10], v[11]);
    dft4(v[12], v[13], v[14], v[15]);
    double2 o[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++)
#pragma unroll
        for (int k2 = 0; k2 < 4; k2++)
            o[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
    for (int i = 0; i < 16; i++)
        v[i] = o[i];
}

// One Stockham pass of radix R (power of two) over `rows` transforms of length
// L: butterfly j of a row reads in[j + r L/R], applies exp(-2 pi i k r / (ns R))
// (k = j mod ns; table tw[k R + r]), and writes out[(j - k) R + k + r ns].
template <int R>
__global__ void __launch_bounds__(PASS_THREADS)
    pass_pow2_kernel(const double2 *__restrict__ in, double2 *__restrict__ out,
                     const double2 *__restrict__ tw, unsigned L, unsigned ns, unsigned total)
{
    const unsigned nb = L / R;
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned f = blockIdx.x * blockDim.x + threadIdx.x; f < total; f += stride) {
        const unsigned p = f / nb, j = f - p * nb;
        const unsigned k = j % ns;
        const double2 *src = in + (size_t)p * L + j;
        double2 v[R];
#pragma unroll
        for (int r = 0; r < R; r++)
            v[r] = src[(size_t)r * nb];
        if (ns > 1) {
            const double2 *t = tw + (size_t)k * R;
#pragma unroll
            for (int r = 1; r < R; r++)
                v[r] = cmul(v[r], __ldg(t + r));
        }
        dft<R>(v);
        double2 *dst = out + (size_t)p * L + (size_t)(j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; r++)
            dst[(size_t)r * ns] = v[r];
    }
}

// One Stockham pass of odd radix R (3 <= R <= 63): G = PASS_THREADS / R
// butterflies per block.  The twiddled inputs v_r go to shared memory, then
// a_q = v_q + v_{R-q} and b_q = v_q - v_{R-q} (q = 1..h, h = (R-1)/2), then
// thread (g, m) forms C = sum_q a_q cos(2 pi q m / R), S = sum_q b_q
// sin(2 pi q m / R) and writes X_m = v_0 + C - i S and X_{R-m} = v_0 + C + i S
// (m = 0: X_0 = v_0 + sum a_q).  cs[t] = (cos, sin)(2 pi t / R).
__global__ void __launch_bounds__(PASS_THREADS)
    pass_odd_kernel(const double2 *__restrict__ in, double2 *__restrict__ out,
                    const double2 *__restrict__ tw, const double2 *__restrict__ cs, unsigned L,
                    unsigned ns, int R, unsigned total)
{
    __shared__ double2 sv[PASS_THREADS];
    __shared__ double2 sab[PASS_THREADS];
    __shared__ double2 scs[64];
    const int h = (R - 1) >> 1;
    const int G = PASS_THREADS / R;
    const unsigned nb = L / R;
    const unsigned f0 = blockIdx.x * (unsigned)G;
    const int t = threadIdx.x;
    if (t < R)
        scs[t] = cs[t];
    if (t < G * R) {
        const int g = t / R, r = t - g * R;
        const unsigned f = f0 + g;
        double2 v = make_double2(0.0, 0.0);
        if (f < total) {
            const unsigned p = f / nb, j = f - p * nb;
            v = in[(size_t)p * L + j + (size_t)r * nb];
            if (ns > 1 && r > 0)
                v = cmul(v, __ldg(tw + (size_t)(j % ns) * R + r));
        }
        sv[g * R + r] = v;
    }
    __syncthreads();
    if (t < G * h) {
        const int g = t / h, q = t - g * h + 1;
        const double2 x = sv[g * R + q], y = sv[g * R + R - q];
        sab[g * 2 * h + q - 1] = cadd(x, y);
        sab[g * 2 * h + h + q - 1] = csub(x, y);
    }
    __syncthreads();
    if (t < G * (h + 1)) {
        const int g = t / (h + 1), m = t - g * (h + 1);
        const unsigned f = f0 + g;
        if (f < total) {
            const unsigned p = f / nb, j = f - p * nb;
            const unsigned k = j % ns;
            double2 *dst = out + (size_t)p * L + (size_t)(j - k) * R + k;
            const double2 v0 = sv[g * R];
            const double2 *a = sab + g * 2 * h, *b = a + h;
            // m = 0 runs the same loop (cos 0 = 1, sin 0 = 0: C = sum a_q,
            // S = 0), so the warp does not split on it
            double2 C = make_double2(0.0, 0.0), S = make_double2(0.0, 0.0);
            int idx = 0;
            for (int q = 0; q < h; q++) {
                idx += m;
                idx -= idx >= R ? R : 0;
                const double c = scs[idx].x, s = scs[idx].y;
                C.x = fma(a[q].x, c, C.x);
                C.y = fma(a[q].y, c, C.y);
                S.x = fma(b[q].x, s, S.x);
                S.y = fma(b[q].y, s, S.y);
            }
            const double re = v0.x + C.x, im = v0.y + C.y;
            dst[(size_t)m * ns] = make_double2(re + S.y, im - S.x);
            if (m > 0)
                dst[(size_t)(R - m) * ns] = make_double2(re - S.y, im + S.x);
        }
    }
}

// (cos, sin)(pi x) for x = 2 m / d with the angle reduced to (-pi, pi].
__device__ __forceinline__ double2 unit_root(long long m, long long d)
{
    m %= d;
    if (m < 0)
        m += d;
    if (2 * m > d)
        m -= d;
    double s, c;
    sincospi(2.0 * (double)m / (double)d, &s, &c);
    return make_double2(c, s);
}

// tw[k R + r] = exp(-2 pi i k r / (ns R)), k < ns, r < R
__global__ void twiddle_kernel(double2 *tw, unsigned ns, int R)
{
    const unsigned n = ns * (unsigned)R;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned k = i / R, r = i - k * R;
        const double2 w = unit_root(-(long long)k * r, (long long)n);
        tw[i] = w;
    }
}

// cs[t] = (cos, sin)(2 pi t / R)
__global__ void odd_table_kernel(double2 *cs, int R)
{
    const int t = threadIdx.x;
    if (t < R)
        cs[t] = unit_root(t, R);
}

// w[n] = exp(-i pi n^2 / N) (n^2 reduced mod 2N in integers)
__global__ void chirp_kernel(double2 *w, unsigned N)
{
    for (unsigned n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const unsigned long long q = ((unsigned long long)n * n) % (2ull * N);
        w[n] = unit_root(-(long long)q, 2ll * N);
    }
}

// b[m] = conj w[m] (m < N), b[M - m] = conj w[m] (0 < m < N), 0 elsewhere
__global__ void chirp_filter_kernel(const double2 *w, unsigned N, unsigned M, double2 *b)
{
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        double2 v = make_double2(0.0, 0.0);
        if (i < N)
            v = make_double2(w[i].x, -w[i].y);
        else if (i > M - N)
            v = make_double2(w[M - i].x, -w[M - i].y);
        b[i] = v;
    }
}

// z[p][n] = (d_{2p}[n] + i d_{2p+1}[n]) (times w[n] for Bluestein; 0 for
// n >= N), d = exp(-scale tau) inv_mean - 1; a missing second row counts as 0.
__global__ void power_pack_kernel(const double *__restrict__ tau, unsigned rows, unsigned N,
                                  unsigned L, double scale, double inv_mean,
                                  const double2 *__restrict__ chirp,
                                  const double *__restrict__ etab, double2 *__restrict__ z,
                                  unsigned total)
{
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const unsigned p = i / L, n = i - p * L;
        double2 v = make_double2(0.0, 0.0);
        if (n < N) {
            const size_t ra = 2 * (size_t)p;
            v.x = fma(fexp(-scale * tau[ra * N + n], etab), inv_mean, -1.0);
            if (ra + 1 < rows)
                v.y = fma(fexp(-scale * tau[(ra + 1) * N + n], etab), inv_mean, -1.0);
            if (chirp)
                v = cmul(v, chirp[n]);
        }
        z[i] = v;
    }
}

// a[p][m] = conj(a[p][m] bhat[m])
__global__ void filter_conj_kernel(double2 *a, const double2 *__restrict__ bhat, unsigned L,
                                   unsigned total)
{
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const double2 v = cmul(a[i], bhat[i % L]);
        a[i] = make_double2(v.x, -v.y);
    }
}

// partial[s][k] = sum over the pairs of segment s, in order, of
// |Z_k|^2 + |Z_{(N-k) mod N}|^2.
__global__ void power_partial_kernel(const double2 *__restrict__ Z, unsigned pairs, unsigned L,
                                     unsigned N, unsigned nk, double *partial)
{
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk)
        return;
    const unsigned s = blockIdx.y;
    const unsigned p0 = (unsigned)((unsigned long long)pairs * s / POWER_SEGMENTS);
    const unsigned p1 = (unsigned)((unsigned long long)pairs * (s + 1) / POWER_SEGMENTS);
    const unsigned k2 = k == 0 ? 0 : N - k;
    double sum = 0.0;
#pragma unroll 4
    for (unsigned p = p0; p < p1; p++) {
        const double2 a = Z[(size_t)p * L + k], b = Z[(size_t)p * L + k2];
        sum += fma(a.x, a.x, a.y * a.y) + fma(b.x, b.x, b.y * b.y);
    }
    partial[(size_t)s * nk + k] = sum;
}

// power[k] += factor * sum over segments (in order) of partial[s][k]
__global__ void power_combine_kernel(const double *partial, unsigned nk, double factor,
                                     double *power)
{
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk)
        return;
    double sum = 0.0;
    for (int s = 0; s < POWER_SEGMENTS; s++)
        sum += partial[(size_t)s * nk + k];
    power[k] += factor * sum;
}

std::vector<long long> prime_factors(long long n)
{
    std::vector<long long> f;
    for (long long p = 2; p * p <= n; p++)
        while (n % p == 0) {
            f.push_back(p);
            n /= p;
        }
    if (n > 1)
        f.push_back(n);
    return f;
}

// smallest 2^a 3^b 5^c 7^d >= m
long long smooth7_at_least(long long m)
{
    long long best = -1;
    for (long long a = 1; a < 2 * m; a *= 2)
        for (long long b = a; b < 2 * m; b *= 3)
            for (long long c = b; c < 2 * m; c *= 5)
                for (long long d = c; d < 2 * m; d *= 7)
                    if (d >= m && (best < 0 || d < best))
                        best = d;
    return best;
}

unsigned grid_for(unsigned long long n, int threads)
{
    const unsigned long long b = (n + threads - 1) / threads;
    return (unsigned)(b < 1 ? 1 : (b > 65535ull * 32 ? 65535ull * 32 : b));
}

// Runs the plan's passes on `rows` transforms in x (scratch y); returns the
// buffer that holds the result.
double2 *run_passes(const PowerPlan &pl, const double2 *tables, double2 *x, double2 *y,
                    unsigned rows, cudaStream_t s, int &launches)
{
    const unsigned L = (unsigned)pl.len;
    for (const PowerPass &ps : pl.passes) {
        const unsigned total = rows * (L / ps.radix);
        const double2 *tw = tables + ps.tw_off;
        const unsigned ns = (unsigned)ps.ns;
        switch (ps.radix) {
        case 2:
            pass_pow2_kernel<2><<<grid_for(total, PASS_THREADS), PASS_THREADS, 0, s>>>(
                x, y, tw, L, ns, total);
            break;
        case 4:
            pass_pow2_kernel<4><<<grid_for(total, PASS_THREADS), PASS_THREADS, 0, s>>>(
                x, y, tw, L, ns, total);
            break;
        case 8:
            pass_pow2_kernel<8><<<grid_for(total, PASS_THREADS), PASS_THREADS, 0, s>>>(
                x, y, tw, L, ns, total);
            break;
        case 16:
            pass_pow2_kernel<16><<<grid_for(total, PASS_THREADS), PASS_THREADS, 0, s>>>(
                x, y, tw, L, ns, total);
            break;
        default: {
            const unsigned G = PASS_THREADS / ps.radix;
            const unsigned blocks = (total + G - 1) / G;
            pass_odd_kernel<<<blocks, PASS_THREADS, 0, s>>>(x, y, tw, tables + ps.cs_off, L, ns,
                                                           ps.radix, total);
        }
        }
        launches++;
        std::swap(x, y);
    }
    return x;
}

}  // namespace

PowerPlan power_plan(long long npix)
{
    PowerPlan pl;
    pl.npix = npix;
    const std::vector<long long> f = prime_factors(npix);
    long long pmax = 1;
    for (long long p : f)
        pmax = p > pmax ? p : pmax;
    pl.bluestein = pmax > POWER_MAX_ODD_RADIX;
    pl.len = pl.bluestein ? smooth7_at_least(2 * npix - 1) : npix;
    std::vector<long long> g = prime_factors(pl.len);
    int twos = 0;
    std::vector<int> radix;
    for (long long p : g)
        if (p == 2)
            twos++;
        else
            radix.push_back((int)p);
    std::vector<int> order;
    for (; twos >= 4; twos -= 4)
        order.push_back(16);
    if (twos)
        order.push_back(1 << twos);
    order.insert(order.end(), radix.begin(), radix.end());
    long long ns = 1, off = 0;
    for (int r : order) {
        PowerPass ps;
        ps.radix = r;
        ps.ns = ns;
        ps.tw_off = off;
        off += ns * r;
        ps.cs_off = -1;
        if (r & 1) {
            ps.cs_off = off;
            off += r;
        }
        pl.passes.push_back(ps);
        ns *= r;
    }
    pl.table_len = off;
    return pl;
}

int power_plan_tables(const PowerPlan &pl, double2 *tables, double2 *chirp, double2 *bhat,
                      double2 *scratch, cudaStream_t s)
{
    int launches = 0;
    for (const PowerPass &ps : pl.passes) {
        if (ps.ns > 1) {
            twiddle_kernel<<<grid_for((unsigned long long)ps.ns * ps.radix, 256), 256, 0, s>>>(
                tables + ps.tw_off, (unsigned)ps.ns, ps.radix);
            launches++;
        }
        if (ps.cs_off >= 0) {
            odd_table_kernel<<<1, 64, 0, s>>>(tables + ps.cs_off, ps.radix);
            launches++;
        }
    }
    if (pl.bluestein) {
        const unsigned N = (unsigned)pl.npix, M = (unsigned)pl.len;
        chirp_kernel<<<grid_for(N, 256), 256, 0, s>>>(chirp, N);
        chirp_filter_kernel<<<grid_for(M, 256), 256, 0, s>>>(chirp, N, M, scratch);
        launches += 2;
        const double2 *r = run_passes(pl, tables, scratch, bhat, 1, s, launches);
        if (r != bhat) {
            cudaMemcpyAsync(bhat, r, sizeof(double2) * M, cudaMemcpyDeviceToDevice, s);
        }
    }
    return launches;
}

long long power_pairs_per_chunk(const PowerPlan &pl, long long nspec)
{
    const long long pairs = (nspec + 1) / 2;
    long long c = (512ll << 20) / (16 * pl.len);
    c = c < 1 ? 1 : c;
    return c < pairs ? c : pairs;
}

int power_chunk(const PowerPlan &pl, const double2 *tables, const double2 *chirp,
                const double2 *bhat, const double *etab, const double *tau, long long rows,
                double scale, double inv_mean, double vmax, double2 *a, double2 *b,
                double *partial, double *power, cudaStream_t s)
{
    int launches = 0;
    const unsigned N = (unsigned)pl.npix, L = (unsigned)pl.len;
    const unsigned pairs = (unsigned)((rows + 1) / 2);
    const unsigned total = pairs * L;
    power_pack_kernel<<<grid_for(total, 256), 256, 0, s>>>(
        tau, (unsigned)rows, N, L, scale, inv_mean, pl.bluestein ? chirp : nullptr, etab, a,
        total);
    launches++;
    double2 *r = run_passes(pl, tables, a, b, pairs, s, launches);
    double norm = 1.0 / ((double)N * (double)N);
    if (pl.bluestein) {
        filter_conj_kernel<<<grid_for(total, 256), 256, 0, s>>>(r, bhat, L, total);
        launches++;
        r = run_passes(pl, tables, r, r == a ? b : a, pairs, s, launches);
        norm /= (double)L * (double)L;
    }
    const unsigned nk = N / 2 + 1;
    power_partial_kernel<<<dim3((nk + 127) / 128, POWER_SEGMENTS), 128, 0, s>>>(r, pairs, L, N,
                                                                              nk, partial);
    power_combine_kernel<<<(nk + 127) / 128, 128, 0, s>>>(partial, nk, 0.5 * vmax * norm,
                                                          power);
    launches += 2;
    return launches;
}

size_t power_partials(long long npix) { return (size_t)POWER_SEGMENTS * (npix / 2 + 1); }

}  // namespace fsg
