// Pair-parallel deposit of optical depth (tau) and column density (colden):
// the replacement for ParticleInterp::compute_tau / compute_colden
// (fake_spectra/part_int.cpp:20-84), LineAbsorption::add_tau_particle /
// add_colden_particle (absorption.cpp:167-279) and SingleAbsorber
// (singleabs.h:63-175).
//
// Work decomposition: one CTA owns one sightline at a time (sightlines are
// visited in descending pair count); each warp takes one (particle,
// sightline) pair at a time and walks its pixel window 32 pixels per step.
// tau: forward from zmax and backward from zmax-1, each direction stopping
// after the first pixel whose contribution is below tautail (that pixel is
// still added) or after nbins/2 pixels, exactly the rule of
// absorption.cpp:250-278; the warp finds the stop lane with a ballot.
// colden: the fixed pixel range of absorption.cpp:190-209.
//
// Accumulation: every contribution is converted to a 128-bit two's-complement
// fixed-point integer with a per-sightline scale 2^S, S chosen from an upper
// bound of that sightline's total so nothing can overflow, and added with
// 64-bit integer atomics (low word + carry into the high word).  Integer
// addition is associative, so the result does not depend on the order in
// which warps and pairs arrive: the output is bitwise deterministic, and the
// sum is exact up to the final rounding to double.  Sightlines with a
// non-finite contribution (inf/NaN inputs) are re-run by a plain FP64-atomic
// fallback so that inf/NaN propagate as they do in the reference.
#include "fsg_internal.cuh"
#include "fsg_voigt.cuh"

#include <cfloat>

namespace fsg {

namespace {

constexpr int NGRID = 8;                          // singleabs.h:8
constexpr double PI_D = 3.14159265358979323846;
constexpr double LIGHT_KMS = 2.99792458e10 / 1e5;  // absorption.cpp:26, km/s

// ---------------------------------------------------------------- kernels
__device__ __forceinline__ double cubic_kernel(double q)   // singleabs.h:17-26
{
    const double norm = 32. / 4 / PI_D;
    if (q >= 1)
        return 0;
    if (q < 0.5)
        return norm * (1 - 6 * q * q + 6 * q * q * q);
    const double t = 1. - q;
    return norm * (2 * t * t * t);
}

__device__ __forceinline__ double quintic_kernel(double q)  // singleabs.h:31-42
{
    const double norm = 9. / 40 / PI_D;
    if (q >= 1)
        return 0;
    if (q < (1. / 3))
        return norm * 6 * (11 - 90 * q * q + 405 * q * q * q * q - 405 * q * q * q * q * q);
    if (q < (2. / 3)) {
        const double a = 3. - 3 * q, b = 2. - 3 * q;
        return norm * (a * a * a * a * a - 6 * b * b * b * b * b);
    }
    const double t = 1. - q;
    return norm * (243 * t * t * t * t * t);
}

// Weight of one line-of-sight node in tau_kern_inner (singleabs.h:158-163):
// unknown kernel ids get no weight factor.
__device__ __forceinline__ double node_weight(int kernel, double q)
{
    if (kernel == SPH_CUBIC)
        return cubic_kernel(q);
    if (kernel == SPH_QUINTIC)
        return quintic_kernel(q);
    if (kernel == TOP_HAT)
        return 3. / 4. / PI_D;
    return 1.0;
}

__device__ __forceinline__ double kernel_max(int kernel)
{
    if (kernel == SPH_CUBIC)
        return 32. / 4 / PI_D;
    if (kernel == SPH_QUINTIC)
        return 9. / 40 / PI_D * 66.0;
    if (kernel == TOP_HAT)
        return 3. / 4. / PI_D;
    return 1.0;
}

// absorption.cpp:53-115: line-of-sight integral of the kernel over one pixel
__device__ double kern_frac(int kernel, double zlow, double zhigh, double smooth, double dr2,
                            double zrange)
{
    if (zlow < -zrange)
        zlow = -zrange;
    if (zhigh > zrange)
        zhigh = zrange;
    if (kernel == SPH_CUBIC || kernel == SPH_QUINTIC) {
        if (zlow > zhigh)
            return 0;
        const bool cub = (kernel == SPH_CUBIC);
        double q = sqrt(dr2 + zlow * zlow) / smooth;
        double total = (cub ? cubic_kernel(q) : quintic_kernel(q)) / 2.;
        const double deltaz = (zhigh - zlow) / NGRID;
        for (int i = 1; i < NGRID; ++i) {
            const double zz = i * deltaz + zlow;
            q = sqrt(dr2 + zz * zz) / smooth;
            total += cub ? cubic_kernel(q) : quintic_kernel(q);
        }
        q = sqrt(dr2 + zhigh * zhigh) / smooth;
        total += (cub ? cubic_kernel(q) : quintic_kernel(q)) / 2.;
        return deltaz * total;
    }
    const double d = zhigh - zlow;
    return 3. / 4. / PI_D * (d > 0. ? d : 0.);
}

// ------------------------------------------------- 128-bit fixed point
__device__ __forceinline__ bool to_fixed(double c, int S, unsigned long long &lo,
                                         unsigned long long &hi)
{
    const long long bits = __double_as_longlong(c);
    unsigned long long m = (unsigned long long)bits & 0xFFFFFFFFFFFFFull;
    int e = (int)((bits >> 52) & 0x7FF);
    if (e == 0)
        e = 1;
    else
        m |= (1ull << 52);
    const int sh = e - 1075 + S;
    unsigned long long l, h;
    if (sh >= 0) {
        if (sh > 126 - 53)
            return false;
        if (sh == 0) {
            l = m;
            h = 0;
        } else if (sh < 64) {
            l = m << sh;
            h = m >> (64 - sh);
        } else {
            l = 0;
            h = m << (sh - 64);
        }
    } else {
        const int r = -sh;
        h = 0;
        l = (r > 63) ? 0ull : ((m + (1ull << (r - 1))) >> r);
    }
    if (bits < 0) {
        l = ~l + 1ull;
        h = ~h + (l == 0ull ? 1ull : 0ull);
    }
    lo = l;
    hi = h;
    return true;
}

__device__ __forceinline__ void fixed_add(unsigned long long *lo, unsigned long long *hi, int j,
                                          unsigned long long l, unsigned long long h)
{
    if (l) {
        const unsigned long long old = atomicAdd(&lo[j], l);
        if (old + l < old)
            h += 1ull;
    }
    if (h)
        atomicAdd(&hi[j], h);
}

__device__ __forceinline__ double from_fixed(unsigned long long lo, unsigned long long hi, int S)
{
    const double v = fma((double)(long long)hi, 18446744073709551616.0, (double)lo);
    return scalbn(v, -S);
}

__device__ __forceinline__ int wrap_bin(long long z, int nbins)
{
    long long j = z % nbins;
    if (j < 0)
        j += nbins;
    return (int)j;
}

// ------------------------------------------------------ per-pair state
struct PairInput {
    double dr2;
    float dens, ppos, pvel, temp, smooth;
};

__device__ __forceinline__ PairInput load_pair(const Particles &p, const PairLists &pl,
                                               long long e, int axis, bool tau)
{
    PairInput in;
    const int ip = pl.part[e];
    in.dr2 = pl.dr2[e];
    const long long k = 3ll * ip + axis - 1;
    in.ppos = p.pos[k];
    in.dens = p.dens[ip];
    in.smooth = p.hh[ip];
    if (tau) {
        in.pvel = p.vel[k];
        in.temp = p.temp[ip];
    } else {
        in.pvel = 0.f;
        in.temp = 0.f;
    }
    return in;
}

// SingleAbsorber (singleabs.h:81-90) + the per-particle constants of add_tau_particle
struct TauPair {
    double btherm, half_b, inv_b, aa, vel, ampd, deltav;
    double vv[NGRID - 1], w[NGRID - 1];
    long long zmax;
};

__device__ __forceinline__ bool tau_setup(const LineParams &lp, const PairInput &in, TauPair &s)
{
    const double hh2 = (double)__fmul_rn(in.smooth, in.smooth);
    if (hh2 - in.dr2 <= 0)
        return false;   // absorption.cpp:232
    s.btherm = lp.bfac * sqrt((double)in.temp);
    s.half_b = s.btherm / 2.;
    s.inv_b = 1.0 / s.btherm;
    s.vel = __dadd_rn(__dmul_rn(lp.velfac, (double)in.ppos), (double)in.pvel);
    const double vdr2 = (lp.velfac * in.dr2) * lp.velfac;
    const double vsmooth = lp.velfac * (double)in.smooth;
    s.aa = lp.voigt_fac / s.btherm;
    const double vhigh = (vsmooth * vsmooth > vdr2 ? sqrt(vsmooth * vsmooth - vdr2) : 0);
    s.deltav = 2. * vhigh / NGRID;
#pragma unroll
    for (int i = 1; i < NGRID; ++i) {
        const double vv = i * s.deltav - vhigh;
        s.vv[i - 1] = vv;
        s.w[i - 1] = node_weight(lp.kernel, sqrt(vdr2 + vv * vv) / vsmooth);
    }
    const double amp = lp.sigma_a / sqrt(PI_D) * (LIGHT_KMS / s.btherm);
    s.ampd = amp * (double)in.dens;
    const double bintov = lp.vbox / lp.nbins;
    s.zmax = (long long)floor(s.vel / bintov);
    return true;
}

// tau_kern_inner, singleabs.h:143-167
__device__ __forceinline__ double tau_inner(const TauPair &s, double vouter)
{
    double total = 0;
#pragma unroll
    for (int i = 0; i < NGRID - 1; ++i)
        total += voigt_f64((s.vv[i] - vouter) * s.inv_b, s.aa) * s.w[i];
    return s.deltav * total;
}

// tau_kern_outer, singleabs.h:104-126.  A sub-sample count beyond
// MAX_SUBSAMPLES (b -> 0, where the reference's int conversion overflows)
// returns NaN and raises DEVERR_WINDOW_LIMIT instead of looping.
__device__ __forceinline__ double tau_outer(const TauPair &s, double vlow, double vhigh,
                                           unsigned *dev_err)
{
    if ((vhigh - vlow) < s.half_b)
        return tau_inner(s, (vhigh + vlow) / 2.);
    const double npd = 2 * ceil((vhigh - vlow) / s.half_b / 2) + 1.;
    if (!(npd <= MAX_SUBSAMPLES)) {
        atomicOr(dev_err, (unsigned)DEVERR_WINDOW_LIMIT);
        return __longlong_as_double(0x7ff8000000000000ll);
    }
    const int npoints = (int)npd;
    double total = tau_inner(s, vlow) / 2.;
    const double deltav = (vhigh - vlow) / (npoints - 1);
    for (int i = 1; i < npoints - 1; ++i)
        total += tau_inner(s, i * deltav + vlow);
    total += tau_inner(s, vhigh) / 2.;
    return total / (npoints - 1);
}

// Upper bound of |taulast| for this pair (any pixel): |amp dens/velfac| x
// deltav x 7 x max|kernel weight| x max H, H <= 1 for a >= 0.
__device__ __forceinline__ double tau_pair_bound(const LineParams &lp, const PairInput &in)
{
    const double hh2 = (double)__fmul_rn(in.smooth, in.smooth);
    if (hh2 - in.dr2 <= 0)
        return 0.0;
    const double btherm = lp.bfac * sqrt((double)in.temp);
    const double aa = lp.voigt_fac / btherm;
    const double hmax = aa >= 0 ? 1.0 : 2.0 * exp(aa * aa) + 1.0;
    const double vsmooth = fabs(lp.velfac * (double)in.smooth);
    const double amp = lp.sigma_a / sqrt(PI_D) * (LIGHT_KMS / btherm);
    return fabs(amp * (double)in.dens / lp.velfac) * (2.0 * vsmooth / NGRID) * 7.0 *
           kernel_max(lp.kernel) * hmax * 1.0001;
}

struct ColdenPair {
    double pos1, zrange, hh2;
    long long zlow, zhigh;
};

__device__ __forceinline__ bool colden_setup(const LineParams &lp, const PairInput &in,
                                             double boxtokpc, ColdenPair &c)
{
    c.pos1 = (double)in.ppos;
    c.hh2 = (double)__fmul_rn(in.smooth, in.smooth);
    if (c.hh2 - in.dr2 <= 0)
        return false;   // absorption.cpp:182
    c.zrange = sqrt(c.hh2 - in.dr2);
    const double lo = floor((c.pos1 - c.zrange) / boxtokpc);
    const double hi = ceil((c.pos1 + c.zrange) / boxtokpc);
    if (!(hi - lo < (double)MAX_COLDEN_WINDOW) || !(fabs(lo) < 9e15) || !(fabs(hi) < 9e15)) {
        c.zlow = 0;
        c.zhigh = -1;   // empty window; the caller flags the pair
        return true;
    }
    c.zlow = (long long)lo;
    c.zhigh = (long long)hi;
    return true;
}

__device__ __forceinline__ bool colden_window_ok(const ColdenPair &c)
{
    return c.zhigh >= c.zlow;
}

__device__ __forceinline__ double colden_pair_bound(const LineParams &lp, const PairInput &in,
                                                    double boxtokpc)
{
    ColdenPair c;
    if (!colden_setup(lp, in, boxtokpc, c))
        return 0.0;
    const double npix = (double)(c.zhigh - c.zlow + 1);
    const double wraps = ceil(npix / lp.nbins);
    return fabs((double)in.dens) * kernel_max(lp.kernel) * fabs(boxtokpc) * 1.001 *
           (wraps > 1.0 ? wraps : 1.0);
}

// ------------------------------------------------------------ reductions
__device__ __forceinline__ double block_sum(double v, double *scratch)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0)
        scratch[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    double t = 0;
    for (int i = 0; i < nw; i++)
        t += scratch[i];
    return t;
}

struct DepositArgs {
    LineParams lp;
    LineTables t;
    Particles p;
    PairLists pl;
    const int *line_order;
    int nlos;
    double *out;
    unsigned *ticket;
    int *bad_lines;
    int *n_bad;
    unsigned *dev_err;
    unsigned long long *gacc;   // global accumulators when not in shared memory
    int smem_mode;
    int persistent;
};

// Walk one tau pair with the whole warp.
__device__ __forceinline__ void walk_tau(const DepositArgs &a, const TauPair &s, int S,
                                         unsigned long long *lo, unsigned long long *hi,
                                         int *bad, int lane)
{
    const int nbins = a.lp.nbins;
    const double bintov = a.lp.vbox / nbins;
    const long long half = nbins / 2;
    // forward: z in [zmax, zmax + nbins/2)
    for (int dir = 0; dir < 2; dir++) {
        const long long start = dir == 0 ? s.zmax : s.zmax - 1;
        for (long long step = 0; step < half; step += 32) {
            const long long k = step + lane;
            const bool valid = k < half;
            const long long z = dir == 0 ? start + k : start - k;
            double tl = 0.0;
            bool stop = false;
            if (valid) {
                const double vlow = (double)z * bintov - s.vel;
                tl = s.ampd * tau_outer(s, vlow, vlow + bintov, a.dev_err) / a.lp.velfac;
                stop = tl < a.lp.tautail;
            }
            const unsigned m = __ballot_sync(0xffffffffu, valid && stop);
            const int last = m ? (__ffs(m) - 1) : 31;
            if (valid && lane <= last) {
                if (!isfinite(tl)) {
                    *bad = 1;
                } else {
                    unsigned long long l, h;
                    if (to_fixed(tl, S, l, h))
                        fixed_add(lo, hi, wrap_bin(z, nbins), l, h);
                    else
                        atomicOr(a.dev_err, (unsigned)DEVERR_FIXED_OVERFLOW);
                }
            }
            if (m)
                break;
        }
    }
}

__device__ __forceinline__ void walk_colden(const DepositArgs &a, const PairInput &in,
                                            const ColdenPair &c, double boxtokpc, int S,
                                            unsigned long long *lo, unsigned long long *hi,
                                            int *bad, int lane)
{
    const int nbins = a.lp.nbins;
    for (long long z = c.zlow + lane; z <= c.zhigh; z += 32) {
        const double plow = (boxtokpc * (double)z - c.pos1);
        const double v = (double)in.dens *
                         kern_frac(a.lp.kernel, plow, plow + boxtokpc, (double)in.smooth, in.dr2,
                                   c.zrange);
        if (!isfinite(v)) {
            *bad = 1;
        } else {
            unsigned long long l, h;
            if (to_fixed(v, S, l, h))
                fixed_add(lo, hi, wrap_bin(z, nbins), l, h);
            else
                atomicOr(a.dev_err, (unsigned)DEVERR_FIXED_OVERFLOW);
        }
    }
}

template <bool TAU>
__global__ void __launch_bounds__(256) deposit_kernel(DepositArgs a)
{
    extern __shared__ unsigned long long smem[];
    __shared__ double red[32];
    __shared__ int s_bad;
    __shared__ unsigned s_ticket;
    const int nbins = a.lp.nbins;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const double boxtokpc = a.lp.vbox / nbins / a.lp.velfac;

    unsigned ticket = blockIdx.x;
    if (a.persistent) {
        if (threadIdx.x == 0)
            s_ticket = atomicAdd(a.ticket, 1u);
        __syncthreads();
        ticket = s_ticket;
    }
    while (ticket < (unsigned)a.nlos) {
        const int line = a.line_order[ticket];
        const int axis = a.t.axis[line];
        const long long e0 = a.pl.off[line], e1 = a.pl.off[line + 1];
        // 1. fixed-point scale from an upper bound of the sightline total
        double b = 0.0;
        for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
            const PairInput in = load_pair(a.p, a.pl, e, axis, TAU);
            b += TAU ? tau_pair_bound(a.lp, in) : colden_pair_bound(a.lp, in, boxtokpc);
        }
        const double B = block_sum(b, red);
        if (threadIdx.x == 0)
            s_bad = !isfinite(B);
        unsigned long long *lo, *hi;
        if (a.smem_mode) {
            lo = smem;
            hi = smem + nbins;
        } else {
            lo = a.gacc + (size_t)line * 2 * nbins;
            hi = lo + nbins;
        }
        for (int j = threadIdx.x; j < nbins; j += blockDim.x) {
            lo[j] = 0ull;
            hi[j] = 0ull;
        }
        __syncthreads();
        const int S = (B > 0.0 && !s_bad) ? 124 - ilogb(B) : 0;
        // 2. deposit: warp per pair
        if (!s_bad && B > 0.0) {
            for (long long e = e0 + warp; e < e1; e += nwarps) {
                const PairInput in = load_pair(a.p, a.pl, e, axis, TAU);
                if (TAU) {
                    TauPair s;
                    if (tau_setup(a.lp, in, s))
                        walk_tau(a, s, S, lo, hi, &s_bad, lane);
                } else {
                    ColdenPair c;
                    if (colden_setup(a.lp, in, boxtokpc, c)) {
                        if (!colden_window_ok(c)) {
                            if (lane == 0)
                                atomicOr(a.dev_err, (unsigned)DEVERR_WINDOW_LIMIT);
                            s_bad = 1;
                        } else {
                            walk_colden(a, in, c, boxtokpc, S, lo, hi, &s_bad, lane);
                        }
                    }
                }
            }
        }
        __syncthreads();
        // 3. flush (rows are owned by this CTA: plain coalesced stores)
        if (s_bad) {
            if (threadIdx.x == 0)
                a.bad_lines[atomicAdd(a.n_bad, 1)] = line;
        } else if (B > 0.0) {
            double *row = a.out + (size_t)line * nbins;
            for (int j = threadIdx.x; j < nbins; j += blockDim.x)
                row[j] = from_fixed(lo[j], hi[j], S);
        }
        if (!a.persistent)
            break;
        __syncthreads();
        if (threadIdx.x == 0)
            s_ticket = atomicAdd(a.ticket, 1u);
        __syncthreads();
        ticket = s_ticket;
    }
}

// Fallback for sightlines with non-finite contributions: FP64 atomics straight
// into the output row, so inf and NaN combine as the reference's += does.
template <bool TAU>
__global__ void __launch_bounds__(256) fallback_kernel(LineParams lp, LineTables t, Particles p,
                                                       PairLists pl, const int *bad_lines,
                                                       double *out, unsigned *dev_err)
{
    const int line = bad_lines[blockIdx.x];
    const int axis = t.axis[line];
    const int nbins = lp.nbins;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const double boxtokpc = lp.vbox / nbins / lp.velfac;
    double *row = out + (size_t)line * nbins;
    const long long e0 = pl.off[line], e1 = pl.off[line + 1];
    for (long long e = e0 + warp; e < e1; e += nwarps) {
        const PairInput in = load_pair(p, pl, e, axis, TAU);
        if (TAU) {
            TauPair s;
            if (!tau_setup(lp, in, s))
                continue;
            const double bintov = lp.vbox / nbins;
            const long long half = nbins / 2;
            for (int dir = 0; dir < 2; dir++) {
                const long long start = dir == 0 ? s.zmax : s.zmax - 1;
                for (long long step = 0; step < half; step += 32) {
                    const long long k = step + lane;
                    const bool valid = k < half;
                    const long long z = dir == 0 ? start + k : start - k;
                    double tl = 0.0;
                    bool stop = false;
                    if (valid) {
                        const double vlow = (double)z * bintov - s.vel;
                        tl = s.ampd * tau_outer(s, vlow, vlow + bintov, dev_err) / lp.velfac;
                        stop = tl < lp.tautail;
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, valid && stop);
                    const int last = m ? (__ffs(m) - 1) : 31;
                    if (valid && lane <= last)
                        atomicAdd(&row[wrap_bin(z, nbins)], tl);
                    if (m)
                        break;
                }
            }
        } else {
            ColdenPair c;
            if (!colden_setup(lp, in, boxtokpc, c))
                continue;
            if (!colden_window_ok(c)) {
                if (lane == 0)
                    atomicOr(dev_err, (unsigned)DEVERR_WINDOW_LIMIT);
                continue;
            }
            for (long long z = c.zlow + lane; z <= c.zhigh; z += 32) {
                const double plow = (boxtokpc * (double)z - c.pos1);
                atomicAdd(&row[wrap_bin(z, nbins)],
                          (double)in.dens * kern_frac(lp.kernel, plow, plow + boxtokpc,
                                                      (double)in.smooth, in.dr2, c.zrange));
            }
        }
    }
}

int g_max_smem_optin = -1;

}  // namespace

int deposit_max_smem_bins()
{
    if (g_max_smem_optin < 0) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        g_max_smem_optin = v;
    }
    // static shared memory of the kernel is < 1 KiB
    return (g_max_smem_optin - 1024) / 16;
}

void launch_deposit(const LineParams &lp, const LineTables &t, const Particles &p,
                    const PairLists &pl, const int *line_order, int nlos, double *out,
                    unsigned *ticket, int *bad_lines, int *n_bad, unsigned *dev_err,
                    unsigned long long *gacc, const DepositLaunch &cfg, cudaStream_t s)
{
    if (nlos == 0)
        return;
    DepositArgs a;
    a.lp = lp;
    a.t = t;
    a.p = p;
    a.pl = pl;
    a.line_order = line_order;
    a.nlos = nlos;
    a.out = out;
    a.ticket = ticket;
    a.bad_lines = bad_lines;
    a.n_bad = n_bad;
    a.dev_err = dev_err;
    a.gacc = gacc;
    a.smem_mode = cfg.smem_mode;
    a.persistent = cfg.persistent;
    const size_t smem = cfg.smem_mode ? (size_t)16 * lp.nbins : 0;
    const int grid = cfg.persistent ? cfg.grid : nlos;
    const int threads = cfg.threads > 0 ? cfg.threads : 256;
    if (lp.compute_tau) {
        cudaFuncSetAttribute(deposit_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        deposit_kernel<true><<<grid, threads, smem, s>>>(a);
    } else {
        cudaFuncSetAttribute(deposit_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        deposit_kernel<false><<<grid, threads, smem, s>>>(a);
    }
}

void launch_deposit_fallback(const LineParams &lp, const LineTables &t, const Particles &p,
                             const PairLists &pl, const int *bad_lines, int n_bad, double *out,
                             unsigned *dev_err, cudaStream_t s)
{
    if (n_bad <= 0)
        return;
    if (lp.compute_tau)
        fallback_kernel<true><<<n_bad, 256, 0, s>>>(lp, t, p, pl, bad_lines, out, dev_err);
    else
        fallback_kernel<false><<<n_bad, 256, 0, s>>>(lp, t, p, pl, bad_lines, out, dev_err);
}

}  // namespace fsg
