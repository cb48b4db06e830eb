// Pair-parallel deposit of optical depth (tau) and column density (colden):
// the replacement for ParticleInterp::compute_tau / compute_colden
// (fake_spectra/part_int.cpp:20-84), LineAbsorption::add_tau_particle /
// add_colden_particle (absorption.cpp:167-279) and SingleAbsorber
// (singleabs.h:63-175).
//
// Work decomposition: one CTA owns one sightline at a time (sightlines are
// visited in descending pair count, either one CTA per sightline or resident
// CTAs draining a ticket queue); each warp takes one (particle, sightline)
// pair at a time and walks its pixel window 32 pixels per step.
// tau: forward from zmax and backward from zmax-1, each direction stopping
// after the first pixel whose contribution is below tautail (that pixel is
// still added) or after nbins/2 pixels, exactly the rule of
// absorption.cpp:250-278; the warp finds the stop lane with a ballot.
// colden: the fixed pixel range of absorption.cpp:190-209.
//
// Two arithmetic forms share this skeleton:
//   FP64 (plain): every quantity in double, as the reference computes it.
//   FP32 (tuned): profile, kernel and pixel arithmetic in float; double only
//     for the particle velocity, the bin of the particle (zmax) and the offset
//     of the first pixel from it, so box-sized coordinates lose nothing.  Far
//     in the damping wing it deposits through per-tile Chebyshev nodes instead
//     of pixel by pixel (see "far-field tiles").
//
// Accumulation: every contribution is converted to a 128-bit two's-complement
// fixed-point integer with a per-sightline scale 2^S, S chosen from an upper
// bound of that sightline's total so nothing can overflow, and added with
// 64-bit integer atomics (low word + carry into the high word) into
// per-sightline accumulators in shared memory.  Integer addition is
// associative, so the result does not depend on the order in which warps and
// pairs arrive: the output is bitwise deterministic and the sum is exact up to
// the final rounding to double.  Sightlines with a non-finite contribution
// (inf/NaN inputs) are re-run by a plain FP64-atomic fallback so that inf/NaN
// propagate as they do in the reference.
#include "fsg_internal.cuh"
#include "fsg_voigt.cuh"

#include <type_traits>

namespace fsg {

namespace {

constexpr int NGRID = 8;                           // singleabs.h:8
constexpr int NODES = NGRID - 1;                   // interior nodes of tau_kern_inner
constexpr double PI_D = 3.14159265358979323846;
constexpr double LIGHT_KMS = 2.99792458e10 / 1e5;  // absorption.cpp:26, in km/s

// ------------------------------------------------------------ SPH kernels
template <class T>
__device__ __forceinline__ T cubic_kernel(T q)   // singleabs.h:17-26
{
    const T norm = (T)(32. / 4 / PI_D);
    if (q >= (T)1)
        return (T)0;
    if (q < (T)0.5)
        return norm * ((T)1 - (T)6 * q * q + (T)6 * q * q * q);
    const T t = (T)1 - q;
    return norm * ((T)2 * t * t * t);
}

template <class T>
__device__ __forceinline__ T quintic_kernel(T q)  // singleabs.h:31-42
{
    const T norm = (T)(9. / 40 / PI_D);
    if (q >= (T)1)
        return (T)0;
    if (q < (T)(1. / 3))
        return norm * (T)6 *
               ((T)11 - (T)90 * q * q + (T)405 * q * q * q * q - (T)405 * q * q * q * q * q);
    if (q < (T)(2. / 3)) {
        const T a = (T)3 - (T)3 * q, b = (T)2 - (T)3 * q;
        return norm * (a * a * a * a * a - (T)6 * b * b * b * b * b);
    }
    const T t = (T)1 - q;
    return norm * ((T)243 * t * t * t * t * t);
}

// FP64 forms with every product and sum rounded on its own (no fused
// multiply-add), in the reference's order of operations.  Near the edge of the
// kernel support, 1 - q cancels and amplifies the last-bit difference a fused
// operation makes (up to 1e-9 relative in a column-density pixel fed only by
// such tails); unfused, each contribution equals the reference's double
// arithmetic.
__device__ __forceinline__ double cubic_kernel_rn(double q)   // singleabs.h:17-26
{
    const double norm = 32. / 4 / PI_D;
    if (q >= 1.0)
        return 0.0;
    if (q < 0.5) {
        const double q6 = __dmul_rn(6.0, q), q6q = __dmul_rn(q6, q);
        return __dmul_rn(norm, __dadd_rn(__dsub_rn(1.0, q6q), __dmul_rn(q6q, q)));
    }
    const double t = __dsub_rn(1.0, q);
    return __dmul_rn(norm, __dmul_rn(__dmul_rn(__dmul_rn(2.0, t), t), t));
}

__device__ __forceinline__ double quintic_kernel_rn(double q)   // singleabs.h:31-42
{
    const double norm = 9. / 40 / PI_D;
    if (q >= 1.0)
        return 0.0;
    if (q < 1. / 3) {
        const double q90 = __dmul_rn(__dmul_rn(90.0, q), q);
        const double q405_4 = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(405.0, q), q), q), q);
        const double q405_5 = __dmul_rn(q405_4, q);
        const double r = __dsub_rn(__dadd_rn(__dsub_rn(11.0, q90), q405_4), q405_5);
        return __dmul_rn(__dmul_rn(norm, 6.0), r);
    }
    if (q < 2. / 3) {
        const double a = __dsub_rn(3.0, __dmul_rn(3.0, q)), b = __dsub_rn(2.0, __dmul_rn(3.0, q));
        const double a5 = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(a, a), a), a), a);
        const double b5 = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(6.0, b), b), b), b), b);
        return __dmul_rn(norm, __dsub_rn(a5, b5));
    }
    const double t = __dsub_rn(1.0, q);
    return __dmul_rn(norm, __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(243.0, t), t), t), t),
                                     t));
}

// Weight of one line-of-sight node in tau_kern_inner (singleabs.h:158-163):
// unknown kernel ids get no weight factor.
template <class T>
__device__ __forceinline__ T node_weight(int kernel, T q)
{
    if (kernel == SPH_CUBIC)
        return cubic_kernel<T>(q);
    if (kernel == SPH_QUINTIC)
        return quintic_kernel<T>(q);
    if (kernel == TOP_HAT)
        return (T)(3. / 4. / PI_D);
    return (T)1;
}

template <>
__device__ __forceinline__ double node_weight<double>(int kernel, double q)
{
    if (kernel == SPH_CUBIC)
        return cubic_kernel_rn(q);
    if (kernel == SPH_QUINTIC)
        return quintic_kernel_rn(q);
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
template <class T>
__device__ T kern_frac(int kernel, T zlow, T zhigh, T smooth, T dr2, T zrange)
{
    if (zlow < -zrange)
        zlow = -zrange;
    if (zhigh > zrange)
        zhigh = zrange;
    if (kernel == SPH_CUBIC || kernel == SPH_QUINTIC) {
        if (zlow > zhigh)
            return (T)0;
        const bool cub = (kernel == SPH_CUBIC);
        T q = sqrt(dr2 + zlow * zlow) / smooth;
        T total = (cub ? cubic_kernel<T>(q) : quintic_kernel<T>(q)) / (T)2;
        const T deltaz = (zhigh - zlow) / (T)NGRID;
        for (int i = 1; i < NGRID; ++i) {
            const T zz = (T)i * deltaz + zlow;
            q = sqrt(dr2 + zz * zz) / smooth;
            total += cub ? cubic_kernel<T>(q) : quintic_kernel<T>(q);
        }
        q = sqrt(dr2 + zhigh * zhigh) / smooth;
        total += (cub ? cubic_kernel<T>(q) : quintic_kernel<T>(q)) / (T)2;
        return deltaz * total;
    }
    const T d = zhigh - zlow;
    if (kernel == VORONOI)   // arepo_kern_frac, absorption.cpp:129-134: overlap length
        return d > (T)0 ? d : (T)0;
    return (T)(3. / 4. / PI_D) * (d > (T)0 ? d : (T)0);
}

// FP64: unfused, in the reference's order (see cubic_kernel_rn)
template <>
__device__ double kern_frac<double>(int kernel, double zlow, double zhigh, double smooth,
                                    double dr2, double zrange)
{
    if (zlow < -zrange)
        zlow = -zrange;
    if (zhigh > zrange)
        zhigh = zrange;
    if (kernel == SPH_CUBIC || kernel == SPH_QUINTIC) {
        if (zlow > zhigh)
            return 0.0;
        const bool cub = (kernel == SPH_CUBIC);
        const auto kern = [cub](double z, double dr2_, double smooth_) {
            const double q = __ddiv_rn(__dsqrt_rn(__dadd_rn(dr2_, __dmul_rn(z, z))), smooth_);
            return cub ? cubic_kernel_rn(q) : quintic_kernel_rn(q);
        };
        double total = kern(zlow, dr2, smooth) / 2.0;
        const double deltaz = __dsub_rn(zhigh, zlow) / NGRID;
        for (int i = 1; i < NGRID; ++i) {
            const double zz = __dadd_rn(__dmul_rn((double)i, deltaz), zlow);
            total = __dadd_rn(total, kern(zz, dr2, smooth));
        }
        total = __dadd_rn(total, kern(zhigh, dr2, smooth) / 2.0);
        return __dmul_rn(deltaz, total);
    }
    const double d = __dsub_rn(zhigh, zlow);
    if (kernel == VORONOI)
        return d > 0.0 ? d : 0.0;
    return __dmul_rn(3. / 4. / PI_D, d > 0.0 ? d : 0.0);
}

// ------------------------------------------------- 128-bit fixed point
// value * 2^S as a 128-bit two's-complement integer (round to nearest).
// Returns false if it would not fit in 126 bits.
__device__ __forceinline__ bool mant_to_fixed(unsigned long long m, int sh, bool neg,
                                              unsigned long long &lo, unsigned long long &hi,
                                              int mbits)
{
    unsigned long long l, h;
    if (sh >= 0) {
        if (sh > 126 - mbits)
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
    if (neg) {
        l = ~l + 1ull;
        h = ~h + (l == 0ull ? 1ull : 0ull);
    }
    lo = l;
    hi = h;
    return true;
}

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
    return mant_to_fixed(m, e - 1075 + S, bits < 0, lo, hi, 53);
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

// ------------------------------------------------- split fixed point (FP32 form)
// value * 2^S = hi * 2^32 + lo with lo in [0, 2^32).  The lo limbs and the
// signed hi parts accumulate in two 64-bit words per pixel with no carry
// between them (lo stays below 2^64 for fewer than 2^32 contributions), so each
// add is a fire-and-forget atomic.  S puts the sightline bound B at 2^91, so hi
// stays below 2^60.  The integer sums are exact: results do not depend on the
// order of the adds.
constexpr int SPLIT_TOP = 91;

__device__ __forceinline__ void split_sign(bool neg, unsigned l32, unsigned long long h,
                                           unsigned long long &lo, long long &hi)
{
    if (neg) {   // -(h 2^32 + l) = (-h - [l != 0]) 2^32 + (2^32 - l) mod 2^32
        hi = -(long long)h - (l32 != 0u ? 1 : 0);
        lo = (unsigned long long)(0u - l32);
    } else {
        hi = (long long)h;
        lo = l32;
    }
}

// Returns false if |v| 2^S >= 2^92 (round to nearest, ties away from zero).
__device__ __forceinline__ bool split_from(float v, int S, unsigned long long &lo, long long &hi)
{
    const int bits = __float_as_int(v);
    unsigned m = (unsigned)bits & 0x7FFFFFu;
    int e = (bits >> 23) & 0xFF;
    if (e == 0)
        e = 1;
    else
        m |= 0x800000u;
    const int p = e - 150 + S;   // |v| 2^S = m 2^p, m < 2^24
    unsigned l32;
    unsigned long long h;
    if (p >= 32) {
        if (p > 68)
            return false;
        l32 = 0u;
        h = (unsigned long long)m << (p - 32);
    } else if (p >= 0) {
        const unsigned long long c = (unsigned long long)m << p;
        l32 = (unsigned)c;
        h = c >> 32;
    } else {
        l32 = (p < -25) ? 0u : (((m >> (-p - 1)) + 1u) >> 1);
        h = 0;
    }
    split_sign(bits < 0, l32, h, lo, hi);
    return true;
}

__device__ __forceinline__ bool split_from(double v, int S, unsigned long long &lo, long long &hi)
{
    const long long bits = __double_as_longlong(v);
    unsigned long long m = (unsigned long long)bits & 0xFFFFFFFFFFFFFull;
    int e = (int)((bits >> 52) & 0x7FF);
    if (e == 0)
        e = 1;
    else
        m |= (1ull << 52);
    const int p = e - 1075 + S;   // |v| 2^S = m 2^p, m < 2^53
    unsigned l32;
    unsigned long long h;
    if (p >= 32) {
        if (p > 39)
            return false;
        l32 = 0u;
        h = m << (p - 32);
    } else if (p >= 0) {
        l32 = (unsigned)(m << p);
        h = p == 0 ? (m >> 32) : (m >> (32 - p));
    } else {
        const unsigned long long c = (p < -54) ? 0ull : (((m >> (-p - 1)) + 1ull) >> 1);
        l32 = (unsigned)c;
        h = c >> 32;
    }
    split_sign(bits < 0, l32, h, lo, hi);
    return true;
}

__device__ __forceinline__ void split_add(unsigned long long *lo_acc, unsigned long long *hi_acc,
                                          int j, unsigned long long lo, long long hi)
{
    if (lo)
        atomicAdd(&lo_acc[j], lo);
    if (hi)
        atomicAdd(&hi_acc[j], (unsigned long long)hi);
}

__device__ __forceinline__ double from_split(unsigned long long lo, unsigned long long hi, int S)
{
    const long long h = (long long)hi + (long long)(lo >> 32);
    const double v = fma((double)h, 4294967296.0, (double)(lo & 0xFFFFFFFFull));
    return scalbn(v, -S);
}

__device__ __forceinline__ int wrap_bin(long long z, int nbins)
{
    long long j = z % nbins;
    if (j < 0)
        j += nbins;
    return (int)j;
}

// ------------------------------------------------------ per-pair inputs
struct PairInput {
    double dr2;
    float dens, ppos, pvel, temp, smooth;
};

// A pair naming a particle outside [0, n) (pair lists that do not belong to
// these particles) is flagged and read as an empty pair (h = 0), which every
// deposit skips.
__device__ __forceinline__ PairInput load_pair(const Particles &p, const PairLists &pl,
                                               long long e, int axis, bool tau, unsigned *dev_err)
{
    PairInput in;
    const int ip = pl.part[e];
    in.dr2 = pl.dr2[e];
    if ((unsigned long long)(long long)ip >= (unsigned long long)p.n) {
        atomicOr(dev_err, (unsigned)DEVERR_PAIR_INDEX);
        in.dr2 = 1.0;
        in.ppos = in.dens = in.smooth = in.pvel = in.temp = 0.f;
        return in;
    }
    if (pl.seg) {
        // Voronoi mesh: the cell's segment ends stand in for dr2 and the
        // smoothing length (part_int.cpp:42-43, 75-76)
        const float2 g = pl.seg[e];
        in.dr2 = (double)g.x;
        in.smooth = g.y;
        in.ppos = __ldg(&p.pos[3ll * ip + axis - 1]);
        in.dens = __ldg(&p.dens[ip]);
        if (tau) {
            in.pvel = __ldg(&p.vel[3ll * ip + axis - 1]);
            in.temp = __ldg(&p.temp[ip]);
        } else {
            in.pvel = 0.f;
            in.temp = 0.f;
        }
        return in;
    }
    const long long k = 3ll * ip + axis - 1;
    in.ppos = __ldg(&p.pos[k]);
    in.dens = __ldg(&p.dens[ip]);
    in.smooth = __ldg(&p.hh[ip]);
    if (tau) {
        in.pvel = __ldg(&p.vel[k]);
        in.temp = __ldg(&p.temp[ip]);
    } else {
        in.pvel = 0.f;
        in.temp = 0.f;
    }
    return in;
}

// ------------------------------------------------------ staged pair records
// The FP32 optical-depth deposit reads each pair's particle fields three
// times (two bound passes and the chunk staging).  The first bound pass
// gathers them from the particle arrays once and writes a 32-byte record per
// pair, contiguous in pair order; the second pass reads the records, and each
// warp stages a chunk's records into shared memory with one bulk asynchronous
// copy (cp.async.bulk, completion on an mbarrier) instead of seven scattered
// loads per pair.
struct __align__(16) PairRec {
    float ppos, pvel, temp, smooth;
    float dens;
    int part;
    double dr2;
};
static_assert(sizeof(PairRec) == 32, "PairRec is two 16-byte words");

__device__ __forceinline__ PairRec make_rec(const PairInput &in, int part)
{
    PairRec r;
    r.ppos = in.ppos;
    r.pvel = in.pvel;
    r.temp = in.temp;
    r.smooth = in.smooth;
    r.dens = in.dens;
    r.part = part;
    r.dr2 = in.dr2;
    return r;
}

__device__ __forceinline__ PairInput rec_input(const PairRec &r)
{
    PairInput in;
    in.dr2 = r.dr2;
    in.dens = r.dens;
    in.ppos = r.ppos;
    in.pvel = r.pvel;
    in.temp = r.temp;
    in.smooth = r.smooth;
    return in;
}

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Orders this thread's earlier generic-proxy accesses (to global, or to
// shared memory) before later async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_global()
{
    asm volatile("fence.proxy.async.global;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_shared()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One elected thread: expect `bytes` on the barrier and start the copy of
// `bytes` (a multiple of 16; both addresses 16-byte aligned) from global to
// shared memory; the barrier's phase completes when they have landed.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes,
                                              unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Waits for the barrier phase with parity `parity`; gives up after `tries`
// polls (each poll may suspend the thread for a while) and returns false.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, int tries)
{
    const unsigned a = smem_addr(bar);
    for (int i = 0; i < tries; i++) {
        unsigned done = 0;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (done)
            return true;
    }
    return false;
}
constexpr int STAGE_WAIT_TRIES = 1 << 20;

// Per warp of a deposit block: the barrier of its staged record copies and the
// parity of the phase it waits for next (kept here rather than in registers,
// which the pixel walk needs).
__shared__ unsigned long long s_stage_bar[32];
__shared__ unsigned s_stage_phase[32];

// Work counters of the counting variant (per lane, reduced per CTA at exit):
// a core-branch evals, b wing-branch evals, c other evals, pixels, and d the
// wing evals among b that were summed through the multipole form.
// e, f, g: node-sum samples through the all-wing, all-core and mixed paths
// (the multipole path is d / 7).
struct Counters {
    unsigned long long a = 0, b = 0, c = 0, pixels = 0, d = 0, e = 0, f = 0, g = 0;
};

__device__ __forceinline__ double nan_d() { return __longlong_as_double(0x7ff8000000000000ll); }

// ------------------------------------------------ FP64 (plain form) pair
// SingleAbsorber (singleabs.h:81-90) + the per-particle constants of add_tau_particle
struct Tau64 {
    double btherm, half_b, inv_b, aa, vel, ampd, deltav, bintov, velfac;
    double vv[NODES], w[NODES];
    long long zmax;
    int nbins;

    __device__ __forceinline__ bool setup(const LineParams &lp, const PairInput &in)
    {
        const bool vor = lp.kernel == VORONOI;
        double pos1 = (double)in.ppos;
        if (vor) {
            // absorption.cpp:221-227: segment [dr2, smooth] along the sightline
            const double lim = 2 * lp.vbox / lp.velfac;
            if (in.dr2 > lim || (double)in.smooth > lim)
                return false;
            pos1 = (in.dr2 + (double)in.smooth) / 2.;
        } else {
            const double hh2 = (double)__fmul_rn(in.smooth, in.smooth);
            if (hh2 - in.dr2 <= 0)
                return false;   // absorption.cpp:232
        }
        btherm = lp.bfac * sqrt((double)in.temp);
        half_b = btherm / 2.;
        inv_b = 1.0 / btherm;
        vel = __dadd_rn(__dmul_rn(lp.velfac, pos1), (double)in.pvel);
        const double vdr2 = vor ? lp.velfac * in.dr2 : (lp.velfac * in.dr2) * lp.velfac;
        const double vsmooth = lp.velfac * (double)in.smooth;
        aa = lp.voigt_fac / btherm;
        // node positions and kernel weights unfused, in the reference's order
        // (singleabs.h:85, 150-156; see cubic_kernel_rn)
        const double vs2 = __dmul_rn(vsmooth, vsmooth);
        double vhigh = (vs2 > vdr2 ? __dsqrt_rn(__dsub_rn(vs2, vdr2)) : 0);
        if (vor)   // singleabs.h:85-89
            vhigh = (vdr2 > 0 && vsmooth > 0) ? (vsmooth - vdr2) / 2. : 0.;
        deltav = 2. * vhigh / NGRID;
#pragma unroll
        for (int i = 1; i < NGRID; ++i) {
            const double v = __dsub_rn(__dmul_rn((double)i, deltav), vhigh);
            vv[i - 1] = v;
            w[i - 1] = node_weight<double>(
                lp.kernel, __ddiv_rn(__dsqrt_rn(__dadd_rn(vdr2, __dmul_rn(v, v))), vsmooth));
        }
        const double amp = lp.sigma_a / sqrt(PI_D) * (LIGHT_KMS / btherm);
        ampd = amp * (double)in.dens;
        nbins = lp.nbins;
        bintov = lp.vbox / nbins;
        velfac = lp.velfac;
        zmax = (long long)floor(vel / bintov);
        return true;
    }

    template <bool COUNT>
    __device__ __forceinline__ double inner(double vouter, Counters &ct) const
    {
        double total = 0;
#pragma unroll
        for (int i = 0; i < NODES; ++i) {
            const double u = (vv[i] - vouter) * inv_b;
            if (COUNT) {
                if (aa == 0.0 || aa > 0.1 || aa < 0.0)
                    ct.c++;
                else if (u * u + aa * aa >= 64.0)
                    ct.b++;
                else
                    ct.a++;
            }
            total += voigt_f64(u, aa) * w[i];
        }
        return deltav * total;
    }

    // tau_kern_outer (singleabs.h:104-126); the sub-sample count is capped.
    template <bool COUNT>
    __device__ __forceinline__ double outer(double vlow, double vhigh, unsigned *dev_err,
                                           Counters &ct) const
    {
        if ((vhigh - vlow) < half_b)
            return inner<COUNT>((vhigh + vlow) / 2., ct);
        const double npd = 2 * ceil((vhigh - vlow) / half_b / 2) + 1.;
        if (!(npd <= MAX_SUBSAMPLES)) {
            atomicOr(dev_err, (unsigned)DEVERR_WINDOW_LIMIT);
            return nan_d();
        }
        const int npoints = (int)npd;
        double total = inner<COUNT>(vlow, ct) / 2.;
        const double dv = (vhigh - vlow) / (npoints - 1);
        for (int i = 1; i < npoints - 1; ++i)
            total += inner<COUNT>(i * dv + vlow, ct);
        total += inner<COUNT>(vhigh, ct) / 2.;
        return total / (npoints - 1);
    }

    __device__ __forceinline__ int bin0(int nbins_) const { return wrap_bin(zmax, nbins_); }

    // pixel z = zmax + koff
    template <bool COUNT>
    __device__ __forceinline__ double taulast(int koff, unsigned *dev_err, Counters &ct) const
    {
        const double vlow = (double)(zmax + koff) * bintov - vel;
        return ampd * outer<COUNT>(vlow, vlow + bintov, dev_err, ct) / velfac;
    }
};

// ------------------------------------------------ FP32 (tuned form) pair
// Far-wing multipole form of the 7-node sum.  In the wing every node profile
// is the asymptotic series g(u) = sum_{j=1}^{8} gamma_j u^(-2j) (voigt_wing32,
// gamma_j = a/sqrt(pi) (p_{j-1} - a^2 q_{j-2})).  The nodes are symmetric
// (U_{8-i} = -U_i, equal weights), so with the even moments
// M_m = sum_i w_i U_i^(2m) the binomial expansion of (U_i - V)^(-2j) gives
//   sum_i w_i g(U_i - V) = sum_{r>=1} A_r V^(-2r),
//   A_r = sum_{j=1}^{r} gamma_j C(2r-1, 2r-2j) M_{r-j}.
// With R = 8 terms the truncation error is below 2e-7 relative once
// |V| >= max(3.34 Umax, Umax + 6.5) (Umax = max |U_i|): one Horner polynomial
// per pixel instead of seven profiles.
constexpr int MP_R = 8;

__host__ __device__ constexpr float binom_f(int n, int k)
{
    float r = 1.f;
    for (int i = 1; i <= k; i++)
        r = r * (float)(n - k + i) / (float)i;
    return r;
}

// Per-pair constants of the FP32 form.  One lane computes one pair (the FP64
// parts: the pixel of the particle velocity and its offset, the thermal width,
// the sub-sample count), so a warp sets up 32 pairs for the FP64 cost of one;
// the warp then walks the staged pairs one after another.
constexpr int STAGE_CAREFUL = 1 << 30;   // walk in FP64 (see below)
constexpr int STAGE_SKIP = 1 << 29;      // no overlap (hh^2 <= dr2) or no pair
constexpr int STAGE_TILES = 1 << 28;     // far wing may be deposited per tile (see below)
constexpr int STAGE_NP = (1 << 28) - 1;  // sub-sample count bits

struct __align__(16) Stage32 {
    int j0;                  // bin of pixel zmax = floor(v_particle / pixel width)
    int flags;               // npoints | STAGE_CAREFUL | STAGE_SKIP | STAGE_TILES
    float base0;             // velocity of pixel zmax's low edge - v_particle
    float inv_b;             // 1 / b
    float scale;             // amp dens / velfac x node spacing / (npoints - 1)
    float aa;                // damping parameter a = voigt_fac / b
    float u1;                // node spacing / b: node i sits at U_i = (i - 4) u1
    float vmp;               // |V| beyond which the multipole form holds
    float w[4];              // kernel weights of nodes 1..4 (nodes 5..7 mirror 3..1)
    float A[MP_R];           // far-wing multipole coefficients
};
static_assert(sizeof(Stage32) == 80, "Stage32 is five 16-byte words");

// SingleAbsorber (singleabs.h:81-90) and the per-particle constants of
// add_tau_particle (absorption.cpp:225-247), FP32 form.  Returns false for a
// pair whose smoothing sphere misses the sightline (absorption.cpp:232).
// scale_nod (may be null) receives scale without the density factor.
// Float copies of the line constants the FP32 setup uses (once per sightline).
struct Setup32 {
    float bfac, voigt_fac, ampv, bintov;   // ampv = sigma_a / sqrt(pi) c / velfac
    __device__ __forceinline__ Setup32(const LineParams &lp, double bintov_d)
    {
        bfac = (float)lp.bfac;
        voigt_fac = (float)lp.voigt_fac;
        ampv = (float)(lp.sigma_a / sqrt(PI_D) * LIGHT_KMS / lp.velfac);
        bintov = (float)bintov_d;
    }
};

// The quantities the FP32 form keeps in float (b, a, the amplitude) come
// from float arithmetic (this GPU runs FP64 at 1/64 of the FP32 rate); the
// particle's bin, its offset and the kernel support keep the reference's
// double arithmetic, and so does the sub-sample count where the float ratio
// lies within 1e-5 of one of its decision boundaries (the float ratio is
// within 4e-7 of the double one).
__device__ __forceinline__ bool stage32_setup(const LineParams &lp, const Setup32 &k,
                                              const PairInput &in, double bintov_d,
                                              Stage32 &st, float *scale_nod)
{
    const double hh2 = (double)__fmul_rn(in.smooth, in.smooth);
    if (hh2 - in.dr2 <= 0)
        return false;
    const float b = k.bfac * sqrtf(in.temp);
    const double vel = __dadd_rn(__dmul_rn(lp.velfac, (double)in.ppos), (double)in.pvel);
    const long long zmax = (long long)floor(vel / bintov_d);
    st.j0 = wrap_bin(zmax, lp.nbins);
    st.base0 = (float)((double)zmax * bintov_d - vel);   // FP64 offset of pixel zmax
    st.inv_b = 1.0f / b;
    const float aa = k.voigt_fac * st.inv_b;
    st.aa = aa;
    const bool wide = !(aa >= 0.0f && aa <= 0.1f);
    const float vdr2 = (float)((lp.velfac * in.dr2) * lp.velfac);
    const float vsmooth = (float)(lp.velfac * (double)in.smooth);
    const float vhigh = (vsmooth * vsmooth > vdr2 ? sqrtf(vsmooth * vsmooth - vdr2) : 0.f);
    const float deltav = 2.f * vhigh / NGRID;
#pragma unroll
    for (int i = 1; i <= 4; ++i) {
        const float v = (float)i * deltav - vhigh;
        st.w[i - 1] = node_weight<float>(lp.kernel, sqrtf(vdr2 + v * v) / vsmooth);
    }
    st.u1 = deltav * st.inv_b;
    {
        // even moments M_m = sum_i w_i U_i^(2m): nodes i and 8-i share |U_i| and w_i,
        // the centre node (U = 0) only enters M_0
        const float q1 = st.u1 * st.u1, q2 = 4.f * q1, q3 = 9.f * q1;
        float M[MP_R];
        M[0] = 2.f * (st.w[0] + st.w[1] + st.w[2]) + st.w[3];
        float p1 = st.w[2], p2 = st.w[1], p3 = st.w[0];
#pragma unroll
        for (int m = 1; m < MP_R; m++) {
            p1 *= q1;
            p2 *= q2;
            p3 *= q3;
            M[m] = 2.f * (p1 + p2 + p3);
        }
        const Voigt32 vc = make_voigt32(st.aa);
        const float P[8] = {1.f, 1.5f, 3.75f, 13.125f, 59.0625f, 324.84375f,
                            2111.484375f, 15836.1328125f};
        const float Q[5] = {1.f, 5.f, 26.25f, 157.5f, 1082.8125f};
        float gam[MP_R + 1];
#pragma unroll
        for (int j = 1; j <= MP_R; j++)
            gam[j] = vc.a_sqpi * (P[j - 1] - (j >= 2 && j - 2 < 5 ? vc.a2 * Q[j - 2] : 0.f));
#pragma unroll
        for (int r = 1; r <= MP_R; r++) {
            float acc = 0.f;
#pragma unroll
            for (int j = 1; j <= r; j++)
                acc = fmaf(gam[j] * binom_f(2 * r - 1, 2 * r - 2 * j), M[r - j], acc);
            st.A[r - 1] = acc;
        }
        const float umax = 3.f * fabsf(st.u1);
        st.vmp = fmaxf(3.34f * umax, umax + 6.5f);
    }
    // tau_kern_outer sub-sampling: uniform for the pair (pixel width = bintov):
    // 1 point if bintov < b/2, else 2 ceil(bintov / b) + 1
    const float r = k.bintov * st.inv_b;
    const float rn = (r + 12582912.0f) - 12582912.0f;   // nearest integer (r < 2^22)
    double npd;
    if (fabsf(r - 0.5f) < 1e-5f || (r >= 0.5f && r < 4e6f && fabsf(r - rn) < 1e-5f * r)) {
        const double half_b = lp.bfac * sqrt((double)in.temp) / 2.;
        npd = 1.0;
        if (!(bintov_d < half_b))
            npd = 2 * ceil(bintov_d / half_b / 2) + 1.;
    } else {
        npd = r < 0.5f ? 1.0 : 2.0 * (double)ceilf(r) + 1.0;
    }
    if (!(npd <= MAX_SUBSAMPLES))
        npd = MAX_SUBSAMPLES + 1;   // flagged by the FP64 walk
    const int npoints = (int)npd;
    // Float node offsets keep ~1e-5 absolute accuracy only while |U_i| <= 256;
    // sub-sampled, very narrow or wide (a outside [0, 0.1]) profiles take the
    // FP64 walk.
    const bool careful = wide || npoints > 8 || !(vhigh <= 256.0f * b);
    float sc = k.ampv * st.inv_b * deltav;
    if (npoints > 1)
        sc /= (float)(npoints - 1);
    if (scale_nod)
        *scale_nod = sc;
    st.scale = sc * in.dens;
    // Far-field tiles need a far wing that decreases with |V|: a positive
    // scale and non-negative multipole coefficients (the sum is then
    // increasing in 1/V^2).
    bool mono = !careful && st.scale > 0.f && isfinite(st.scale);
#pragma unroll
    for (int r = 0; r < MP_R; r++)
        mono = mono && st.A[r] >= 0.f && isfinite(st.A[r]);
    st.flags = npoints | (careful ? STAGE_CAREFUL : 0) | (mono ? STAGE_TILES : 0);
    return true;
}

// The FP32 walk of one pair, built from its staged constants (all lanes).
struct Tau32 {
    Voigt32 vc;
    float U[NODES], w[NODES];   // node velocities / b and kernel weights
    float A[MP_R];              // multipole coefficients (far wing)
    float vmp;                  // |V| beyond which the multipole form holds
    float inv_b, base0, bintov, hbin_b, scale, scale_nod, sub_dv;
    float vk, v0, vmid0;        // pixel k: V_low = k vk + v0, V_mid = k vk + vmid0
    float aa_f;
    int j0;
    int npoints;                 // 1: midpoint; else trapezoid points (uniform per pair)
    bool careful;                // walk in FP64 instead (Stage32 flags)
    bool tiles;                  // far wing may be deposited per tile (Stage32 flags)

    __device__ __forceinline__ void load(const Stage32 &st, float bintov_f)
    {
        j0 = st.j0;
        base0 = st.base0;
        inv_b = st.inv_b;
        scale = st.scale;
        scale_nod = 0.f;
        aa_f = st.aa;
        vc = make_voigt32(aa_f);
#pragma unroll
        for (int i = 0; i < NODES; ++i)
            U[i] = (float)(i - 3) * st.u1;
        w[0] = w[6] = st.w[0];
        w[1] = w[5] = st.w[1];
        w[2] = w[4] = st.w[2];
        w[3] = st.w[3];
#pragma unroll
        for (int r = 0; r < MP_R; ++r)
            A[r] = scale * st.A[r];   // inner() returns scaled sums
        vmp = st.vmp;
        bintov = bintov_f;
        hbin_b = 0.5f * bintov * inv_b;
        vk = bintov * inv_b;
        v0 = base0 * inv_b;
        vmid0 = v0 + hbin_b;
        npoints = st.flags & STAGE_NP;
        careful = (st.flags & STAGE_CAREFUL) != 0;
        tiles = (st.flags & STAGE_TILES) != 0 && vk > 0.f;
        sub_dv = npoints > 1 ? __fdividef(bintov, (float)(npoints - 1)) * inv_b : 0.f;
    }

    __device__ __forceinline__ int bin0(int) const { return j0; }

    // scale x the node sum at V (velocity offset / b).  Called by every lane
    // of the warp (lanes past the window compute and discard), so the warp
    // votes below see a converged warp.
    template <bool COUNT>
    __device__ __forceinline__ float inner(float V, const float2 *tab, Counters &ct) const
    {
        if (__all_sync(0xffffffffu, fabsf(V) >= vmp)) {
            const float W = __fdividef(1.0f, V * V);
            float sm = A[MP_R - 1];
#pragma unroll
            for (int r = MP_R - 2; r >= 0; r--)
                sm = fmaf(sm, W, A[r]);
            if (COUNT) {
                ct.b += NODES;
                ct.d += NODES;
            }
            return sm * W;
        }
        return scale * inner_nodes<COUNT>(V, tab, ct);
    }

    template <bool COUNT>
    __device__ __forceinline__ float inner_nodes(float V, const float2 *tab, Counters &ct) const
    {
        float total = 0.f;
        float u[NODES];
        if constexpr (!COUNT) {
            // The node offsets are (i - 3) u1: max_i |U_i - V| = |V| + |U_6|
            // exactly (the same float sum as the farther end node's), and
            // |V| - |U_6| is min_i |U_i - V| once |V| >= |U_6| (a lower bound
            // otherwise).  Three tests instead of three per node.
            const float av = fabsf(V), ext = fabsf(U[NODES - 1]);
            const float near = av - ext, far = av + ext;
#pragma unroll
            for (int i = 0; i < NODES; ++i)
                u[i] = U[i] - V;
            if (__all_sync(0xffffffffu, near >= 6.5f)) {
#pragma unroll
                for (int i = 0; i < NODES; ++i)
                    total = fmaf(voigt_wing32(u[i], vc), w[i], total);
                return total;
            }
            // small damping (uniform over the warp: one pair): the first-order
            // form where every node is inside its table, else per node with
            // the wing form
            if (vc.a <= VOIGT_SMALL_A) {
                if (__all_sync(0xffffffffu, far < VOIGT_SMALL_X)) {
#pragma unroll
                    for (int i = 0; i < NODES; ++i)
                        total = fmaf(voigt_small32(u[i], vc), w[i], total);
                    return total;
                }
#pragma unroll
                for (int i = 0; i < NODES; ++i) {
                    const float h = fabsf(u[i]) < VOIGT_SMALL_X ? voigt_small32(u[i], vc)
                                                                : voigt_wing32(u[i], vc);
                    total = fmaf(h, w[i], total);
                }
                return total;
            }
            if (__all_sync(0xffffffffu, far < 11.9f)) {   // the core form's table ends at 12
#pragma unroll
                for (int i = 0; i < NODES; ++i)
                    total = fmaf(voigt_core32(u[i], vc, tab), w[i], total);
                return total;
            }
            unsigned nn = 0;
#pragma unroll
            for (int i = 0; i < NODES; ++i)
                total = fmaf(voigt_f32<COUNT>(u[i], vc, tab, nn), w[i], total);
            return total;
        }
        // the counting variant: the per-node tests whose paths it counts
        bool wing = true, core = true;
#pragma unroll
        for (int i = 0; i < NODES; ++i) {
            u[i] = U[i] - V;
            wing &= fabsf(u[i]) >= 6.5f;
            core &= fabsf(u[i]) < 11.9f;   // the core form's table ends at 12
        }
        if (__all_sync(0xffffffffu, wing)) {
#pragma unroll
            for (int i = 0; i < NODES; ++i)
                total = fmaf(voigt_wing32(u[i], vc), w[i], total);
            if (COUNT) {
                ct.b += NODES;
                ct.e++;
            }
            return total;
        }
        if (__all_sync(0xffffffffu, core)) {
#pragma unroll
            for (int i = 0; i < NODES; ++i)
                total = fmaf(voigt_core32(u[i], vc, tab), w[i], total);
            if (COUNT) {
                ct.a += NODES;
                ct.f++;
            }
            return total;
        }
        unsigned nn = 0;
#pragma unroll
        for (int i = 0; i < NODES; ++i)
            total = fmaf(voigt_f32<COUNT>(u[i], vc, tab, nn), w[i], total);
        if (COUNT) {
            ct.a += nn;
            ct.b += NODES - nn;
            ct.g++;
        }
        return total;
    }

    // pixel z = zmax + koff; kf == (float)koff, carried by the caller so no
    // int->float conversion runs per pixel
    template <bool COUNT>
    __device__ __forceinline__ float taulast(float kf, unsigned *dev_err, const float2 *tab,
                                             Counters &ct) const
    {
        if (npoints == 1)
            return inner<COUNT>(fmaf(kf, vk, vmid0), tab, ct);
        return trapezoid<COUNT>(fmaf(kf, vk, v0), tab, ct);   // (v_low - v_particle) / b
    }

    template <bool COUNT>
    __device__ __forceinline__ float trapezoid(float vlow_b, const float2 *tab,
                                               Counters &ct) const
    {
        float total = 0.f;
        for (int i = 0; i < npoints; ++i) {
            const float x = i == npoints - 1 ? vlow_b + 2.f * hbin_b : fmaf((float)i, sub_dv, vlow_b);
            const float f = inner<COUNT>(x, tab, ct);
            total = (i == 0 || i == npoints - 1) ? fmaf(0.5f, f, total) : total + f;
        }
        return total;
    }

    // taulast at pixel ka + kb (ka integral; kb = 0 for a pixel, the node's
    // offset for a far-field tile node).  The two-step offset keeps a node's V
    // as accurate as an integral pixel's; with kb = 0 the result is taulast's
    // bit for bit.  One inner() call site keeps the kernel's code small.
    __device__ __forceinline__ float value_at(float ka, float kb, const float2 *tab) const
    {
        Counters ct;
        const float x0 = npoints == 1 ? vmid0 : v0;
        const float x = fmaf(kb, vk, fmaf(ka, vk, x0));
        float total = 0.f;
        const int np = npoints;
        for (int i = 0; i < np; ++i) {
            const float xi = np == 1 ? x : (i == np - 1 ? x + 2.f * hbin_b : fmaf((float)i, sub_dv, x));
            const float f = inner<false>(xi, tab, ct);
            total = (np == 1) ? f : ((i == 0 || i == np - 1) ? fmaf(0.5f, f, total) : total + f);
        }
        return total;
    }

};

// Float constants of tau_pair_bound32 (computed once per thread).
struct Bound32 {
    float bfac, voigt_fac, velfac_abs, ampc, kfac;
    __device__ __forceinline__ explicit Bound32(const LineParams &lp)
    {
        bfac = (float)lp.bfac;
        voigt_fac = (float)lp.voigt_fac;
        velfac_abs = (float)fabs(lp.velfac);
        ampc = (float)(lp.sigma_a / sqrt(PI_D) * LIGHT_KMS / fabs(lp.velfac));
        kfac = (float)(2.0 / NGRID * 7.0 * kernel_max(lp.kernel) * 1.001);
    }
};

// tau_pair_bound in FP32 arithmetic with a 1e-3 margin (the FP32 form's
// contributions are FP32 values too): no FP64 work per pair beyond the overlap
// test, which follows the reference's double comparison.
__device__ __forceinline__ double tau_pair_bound32(const Bound32 &k, const PairInput &in)
{
    const double hh2 = (double)__fmul_rn(in.smooth, in.smooth);
    if (hh2 - in.dr2 <= 0)
        return 0.0;
    const float btherm = k.bfac * sqrtf(in.temp);
    const float aa = k.voigt_fac / btherm;
    const float hmax = aa >= 0.f ? 1.f : 2.f * expf(aa * aa) + 1.f;
    return (double)(fabsf(k.ampc / btherm * in.dens) * (k.velfac_abs * fabsf(in.smooth)) *
                    k.kfac * hmax);
}

// Upper bound of |taulast| for a pair (any pixel): |amp dens/velfac| x deltav x
// 7 x max|kernel weight| x max H, with H <= 1 for a >= 0.
__device__ __forceinline__ double tau_pair_bound(const LineParams &lp, const PairInput &in)
{
    if (lp.kernel == VORONOI) {
        const double lim = 2 * lp.vbox / lp.velfac;
        if (in.dr2 > lim || (double)in.smooth > lim)
            return 0.0;
    } else {
        const double hh2 = (double)__fmul_rn(in.smooth, in.smooth);
        if (hh2 - in.dr2 <= 0)
            return 0.0;
    }
    const double btherm = lp.bfac * sqrt((double)in.temp);
    const double aa = lp.voigt_fac / btherm;
    const double hmax = aa >= 0 ? 1.0 : 2.0 * exp(aa * aa) + 1.0;
    const double vsmooth = fabs(lp.velfac * (double)in.smooth);
    const double amp = lp.sigma_a / sqrt(PI_D) * (LIGHT_KMS / btherm);
    return fabs(amp * (double)in.dens / lp.velfac) * (2.0 * vsmooth / NGRID) * 7.0 *
           kernel_max(lp.kernel) * hmax * 1.0001;
}

// ------------------------------------------------------------ colden pair
// FP32 form of kern_frac for a pixel lying wholly inside the kernel support
// [-zrange, zrange].  Node q values come from the distance d of the node to
// the nearer support edge, anchored in FP64 per pair, so the kernel tails
// (1-q)^3 and (1-q)^5 keep full relative accuracy:
//   1 - q^2 = d (2 zrange - d) / h^2 + (1 - hh2/h^2),   1 - q = (1 - q^2)/(1 + q),
// (hh2 = h*h in float, as the reference forms zrange = sqrt(hh2 - dr2)).
__device__ __forceinline__ float spline_from_eps(bool cubic, float eps)
{
    if (!(eps > 0.f))
        return 0.f;                                  // q >= 1
    const float q2 = fmaxf(1.f - eps, 0.f);
    const float q = sqrtf(q2);
    const float t = eps / (1.f + q);                 // 1 - q without cancellation
    if (cubic) {
        const float norm = (float)(32. / 4 / PI_D);
        if (q < 0.5f)
            return norm * (1.f - 6.f * q2 + 6.f * q2 * q);
        return norm * (2.f * t * t * t);
    }
    const float norm = (float)(9. / 40 / PI_D);
    if (q < (float)(1. / 3)) {
        const float q4 = q2 * q2;
        return norm * 6.f * (11.f - 90.f * q2 + 405.f * q4 - 405.f * q4 * q);
    }
    const float a = 3.f * t, a2 = a * a;
    if (q < (float)(2. / 3)) {
        const float b = a - 1.f, b2 = b * b;
        return norm * (a2 * a2 * a - 6.f * b2 * b2 * b);
    }
    const float t2 = t * t;
    return norm * (243.f * t2 * t2 * t);
}

struct Colden {
    double pos1, zrange, smooth, dr2, boxtokpc, dens;
    float box_f, dL0, dR0, two_zr, inv_h2, ch, dens_f;
    long long zlow, zhigh, kmax;
    int kernel;
    bool ok;   // window within MAX_COLDEN_WINDOW

    __device__ __forceinline__ bool setup(const LineParams &lp, const PairInput &in, double btk)
    {
        pos1 = (double)in.ppos;
        const double hh2 = (double)__fmul_rn(in.smooth, in.smooth);
        if (lp.kernel == VORONOI) {
            // absorption.cpp:170-186: segment [dr2, smooth], centre and half-length
            const double lim = 2 * lp.vbox / lp.velfac;
            if (in.dr2 > lim || (double)in.smooth > lim)
                return false;
            pos1 = (in.dr2 + (double)in.smooth) / 2.;
            zrange = ((double)in.smooth - in.dr2) / 2.;
        } else {
            if (hh2 - in.dr2 <= 0)
                return false;   // absorption.cpp:182
            zrange = sqrt(hh2 - in.dr2);
        }
        boxtokpc = btk;
        smooth = (double)in.smooth;
        dr2 = in.dr2;
        dens = (double)in.dens;
        kernel = lp.kernel;
        const double lo = floor((pos1 - zrange) / boxtokpc);
        const double hi = ceil((pos1 + zrange) / boxtokpc);
        ok = (hi - lo < (double)MAX_COLDEN_WINDOW) && fabs(lo) < 9e15 && fabs(hi) < 9e15;
        zlow = ok ? (long long)lo : 0;
        zhigh = ok ? (long long)hi : -1;
        kmax = zhigh - zlow;
        // FP32 form: edge distances anchored in FP64 at both ends of the window
        box_f = (float)boxtokpc;
        dL0 = (float)(boxtokpc * (double)zlow - pos1 + zrange);    // pixel zlow edge - (-zrange)
        dR0 = (float)(zrange + pos1 - boxtokpc * (double)zhigh);   // zrange - pixel zhigh edge
        two_zr = (float)(2.0 * zrange);
        const double h2 = smooth * smooth;
        inv_h2 = (float)(1.0 / h2);
        ch = (float)((h2 - hh2) / h2);
        dens_f = in.dens;
        return true;
    }

    __device__ __forceinline__ double value64(long long z) const
    {
        const double plow = __dsub_rn(__dmul_rn(boxtokpc, (double)z), pos1);
        return __dmul_rn(dens, kern_frac<double>(kernel, plow, __dadd_rn(plow, boxtokpc), smooth,
                                                 dr2, zrange));
    }
};

__device__ __forceinline__ double colden_pair_bound(const LineParams &lp, const PairInput &in,
                                                    double boxtokpc)
{
    Colden c;
    if (!c.setup(lp, in, boxtokpc))
        return 0.0;
    const double npix = (double)(c.zhigh - c.zlow + 1);
    const double wraps = ceil(npix / lp.nbins);
    return fabs((double)in.dens) * kernel_max(lp.kernel) * fabs(boxtokpc) * 1.001 *
           (wraps > 1.0 ? wraps : 1.0);
}

// Per-pair constants of the FP32 column density (48 bytes), set up by one
// lane per pair like Stage32: the three FP64 edge pixels (first, last two)
// are evaluated here, lane-parallel, and the interior walks in FP32.
constexpr int COL_SKIP = 1, COL_BAD = 2;   // no overlap; window beyond the limit

struct __align__(16) StageCol32 {
    int j0, kmax, flags;
    float dens_f;
    float e0, e1, e2;        // pixels k = 0, kmax - 1, kmax
    float dL0;
    float dR0, two_zr, inv_h2, ch;
};
static_assert(sizeof(StageCol32) == 48, "StageCol32 is three 16-byte words");

__device__ __forceinline__ void stagecol32_setup(const LineParams &lp, const PairInput &in,
                                                 double btk, StageCol32 &st)
{
    Colden c;
    st.flags = 0;
    if (!c.setup(lp, in, btk)) {
        st.flags = COL_SKIP;
        return;
    }
    if (!c.ok) {
        st.flags = COL_BAD;
        return;
    }
    st.j0 = wrap_bin(c.zlow, lp.nbins);
    st.kmax = (int)c.kmax;
    st.dens_f = c.dens_f;
    st.e0 = (float)c.value64(c.zlow);
    st.e1 = c.kmax >= 2 ? (float)c.value64(c.zlow + c.kmax - 1) : 0.f;
    st.e2 = c.kmax >= 1 ? (float)c.value64(c.zhigh) : 0.f;
    st.dL0 = c.dL0;
    st.dR0 = c.dR0;
    st.two_zr = c.two_zr;
    st.inv_h2 = c.inv_h2;
    st.ch = c.ch;
}

// Colden::value32 for an interior pixel 0 < k < kmax - 1 of a staged pair.
__device__ __forceinline__ float colden_interior32(const StageCol32 &st, int kernel, float box_f,
                                                   int k)
{
    if (kernel != SPH_CUBIC && kernel != SPH_QUINTIC)
        return st.dens_f * ((float)(3. / 4. / PI_D) * box_f);
    const bool cubic = (kernel == SPH_CUBIC);
    const float dz = box_f * (1.f / NGRID);
    const float l0 = fmaf((float)k, box_f, st.dL0);
    const float r0 = fmaf((float)(st.kmax - k), box_f, st.dR0);
    float total = 0.f;
#pragma unroll
    for (int i = 0; i <= NGRID; i++) {
        const float d = fminf(fmaf((float)i, dz, l0), fmaf(-(float)i, dz, r0));
        const float eps = fmaf(d * (st.two_zr - d), st.inv_h2, st.ch);
        const float kv = spline_from_eps(cubic, eps);
        total += (i == 0 || i == NGRID) ? 0.5f * kv : kv;
    }
    return st.dens_f * (dz * total);
}

// colden_pair_bound in FP32 with a 1e-3 margin: the window length is bounded
// by 2 zrange / pixel + 3 pixels.
__device__ __forceinline__ double colden_pair_bound32(const LineParams &lp, const PairInput &in,
                                                      float btk_abs, float kfac)
{
    const double hh2 = (double)__fmul_rn(in.smooth, in.smooth);
    if (hh2 - in.dr2 <= 0)
        return 0.0;
    const float zr = sqrtf((float)(hh2 - in.dr2));
    const float npix = 2.f * zr / btk_abs + 3.f;
    const float wraps = fmaxf(1.f, ceilf(npix / (float)lp.nbins));
    return (double)(fabsf(in.dens) * kfac * btk_abs * wraps);
}

// ------------------------------------------------------------ reductions
// Block-wide upper bound of a sightline's total, sum_p b_p over its pairs
// [e0, e1), computed so that it does not depend on how the pairs are spread
// over the threads: with e = max_p ilogb(b_p) (an integer maximum),
//   B = 2^(e - 30) x sum_p ceil(b_p 2^(30 - e)),
// a sum of integers below 2^31 each, exact in 64 bits for up to 2^32 pairs.
// The fixed-point scale follows from ilogb(B), so the output bits are the same
// for every block size, chunk size and queue mode.  Returns +inf when a bound
// is not finite (the sightline then goes to the non-finite fallback) and 0 when
// every bound is 0.  `bound(e)` is evaluated in the first pass and
// `bound_again(e)` (the same value, possibly from a cheaper source) in the
// second; each pair is visited by the same thread in both.
struct BoundScratch {
    int em[32];
    unsigned long long q[32];
};

template <class BoundFn, class AgainFn>
__device__ __forceinline__ double order_free_bound(long long e0, long long e1, BoundFn bound,
                                                   AgainFn bound_again, BoundScratch *sc)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int NONE = -2147483647;
    int em = NONE;
    bool bad = false;
    for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const double b = bound(e);
        if (!isfinite(b))
            bad = true;
        else if (b > 0.0)
            em = max(em, ilogb(b));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        em = max(em, __shfl_xor_sync(0xffffffffu, em, o));
    bad = __any_sync(0xffffffffu, bad);
    __syncthreads();
    if (lane == 0)
        sc->em[warp] = bad ? 2147483647 : em;
    __syncthreads();
    int eall = NONE;
    for (int i = 0; i < nw; i++)
        eall = max(eall, sc->em[i]);
    if (eall == 2147483647)
        return __longlong_as_double(0x7ff0000000000000ll);
    if (eall == NONE)
        return 0.0;
    unsigned long long q = 0;
    for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const double b = bound_again(e);
        if (b > 0.0)
            q += (unsigned long long)ceil(scalbn(b, 30 - eall));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        q += __shfl_xor_sync(0xffffffffu, q, o);
    __syncthreads();
    if (lane == 0)
        sc->q[warp] = q;
    __syncthreads();
    unsigned long long Q = 0;
    for (int i = 0; i < nw; i++)
        Q += sc->q[i];
    return scalbn(__ull2double_ru(Q), eall - 30);
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
    unsigned long long *counters;   // [8] (counting variant only)
    int smem_mode;
    int persistent;
    int chunk;                      // pairs staged per warp (FP32 tau form)
    int tiles;                      // far-field tile accumulators (FP32 tau form)
};

// FMT 0: 128-bit fixed point with carries (FP64 form); 1: split (FP32 form).
template <class R, int FMT>
__device__ __forceinline__ void accumulate(unsigned *dev_err, R v, int j, int S,
                                           unsigned long long *lo, unsigned long long *hi,
                                           int *bad)
{
    if constexpr (FMT == 1 && std::is_same<R, float>::value) {
        // Non-negative finite v with v 2^S = m 2^p, 0 <= p <= 68 (every optical
        // depth contribution: the bound puts the sightline total at 2^91, and a
        // walk stops long before 2^-68 of it): the split_from result without
        // branches.  c = m << min(p, 40) fits in 64 bits (m < 2^24); its low
        // word is lo (zero once p >= 32) and its high word, shifted on by the
        // rest of p, is hi.  Everything else takes the general path below.
        const unsigned fb = __float_as_uint(v);
        if (fb < 0x7F800000u) {
            const unsigned e8 = fb >> 23;
            const unsigned m = (fb & 0x7FFFFFu) | (e8 ? 0x800000u : 0u);
            const int p = (int)(e8 ? e8 : 1u) - 150 + S;
            if ((unsigned)p <= 68u) {
                const int ps = min(p, 40);
                const unsigned long long c = (unsigned long long)m << ps;
                const unsigned l32 = (unsigned)c;
                const unsigned long long h = (c >> 32) << (p - ps);
                if (l32)
                    atomicAdd(&lo[j], (unsigned long long)l32);
                if (h)
                    atomicAdd(&hi[j], h);
                return;
            }
        }
    }
    if (!isfinite(v)) {
        *bad = 1;
        return;
    }
    if constexpr (FMT == 0) {
        unsigned long long l, h;
        if (to_fixed(v, S, l, h))
            fixed_add(lo, hi, j, l, h);
        else
            atomicOr(dev_err, (unsigned)DEVERR_FIXED_OVERFLOW);
    } else {
        unsigned long long l;
        long long h;
        if (split_from(v, S, l, h))
            split_add(lo, hi, j, l, h);
        else
            atomicOr(dev_err, (unsigned)DEVERR_FIXED_OVERFLOW);
    }
}

// bin of pixel zmax + koff from j0 = bin of zmax, |koff| <= nbins
__device__ __forceinline__ int bin_from(int j0, int koff, int nbins)
{
    int j = j0 + koff;
    if (j < 0)
        j += nbins;
    else if (j >= nbins)
        j -= nbins;
    return j;
}

// Walk one tau pair with the whole warp: 32 consecutive pixels per step.
// Pixel offsets from zmax and bins are int32; the FP32 form compares its float
// contribution with tautail in float, so no FP64 work is done per pixel.
template <int PREC, bool COUNT, int FMT, class P>
__device__ __forceinline__ void walk_tau(const DepositArgs &a, const P &s, int S,
                                         unsigned long long *lo, unsigned long long *hi,
                                         int *bad, int lane, const float2 *tab, Counters &ct)
{
    using R = typename std::conditional<PREC == 0, double, float>::type;
    const int nbins = a.lp.nbins;
    const int half = nbins / 2;
    const R tautail = (R)a.lp.tautail;
    const int j0 = s.bin0(nbins);
    const float lane_f = (float)lane;
    for (int dir = 0; dir < 2; dir++) {
        // kf tracks (float)koff exactly (integers below 2^24) without conversions
        float kf = dir == 0 ? lane_f : -1.0f - lane_f;
        const float dkf = dir == 0 ? 32.0f : -32.0f;
        for (int step = 0; step < half; step += 32, kf += dkf) {
            const int k = step + lane;
            const bool valid = k < half;
            const int koff = dir == 0 ? k : -1 - k;
            Counters c1{};
            R tl = (R)0;
            if constexpr (PREC == 0) {
                if (valid)
                    tl = s.template taulast<COUNT>(koff, a.dev_err, c1);
            } else {
                // every lane evaluates (warp-uniform fast paths vote inside)
                tl = s.template taulast<COUNT>(kf, a.dev_err, tab, c1);
            }
            const bool stop = valid && (tl < tautail);
            const unsigned m = __ballot_sync(0xffffffffu, stop);
            const int last = m ? (__ffs(m) - 1) : 31;
            if (valid && lane <= last) {
                accumulate<R, FMT>(a.dev_err, tl, bin_from(j0, koff, nbins), S, lo, hi, bad);
                if (COUNT) {
                    ct.a += c1.a;
                    ct.b += c1.b;
                    ct.c += c1.c;
                    ct.d += c1.d;
                    ct.e += c1.e;
                    ct.f += c1.f;
                    ct.g += c1.g;
                    ct.pixels++;
                }
            }
            if (m)
                break;
        }
    }
}

template <int PREC, bool COUNT>
__device__ __forceinline__ void walk_colden(const DepositArgs &a, const Colden &c, int S,
                                            unsigned long long *lo, unsigned long long *hi,
                                            int *bad, int lane, Counters &ct)
{
    const int nbins = a.lp.nbins;
    const int j0 = wrap_bin(c.zlow, nbins);
    const int kmax = (int)c.kmax;   // < MAX_COLDEN_WINDOW
    static_assert(PREC == 0, "the FP32 column density walks staged pairs");
    for (int k = lane; k <= kmax; k += 32) {
        const int j = (int)(((long long)j0 + k) % nbins);
        accumulate<double, 0>(a.dev_err, c.value64(c.zlow + k), j, S, lo, hi, bad);
        if (COUNT)
            ct.pixels++;
    }
}

// Rare pairs of the FP32 form (see Tau32::careful) walk with the FP64 pair;
// their evaluations count as "other" work.
template <bool COUNT>
__device__ __noinline__ void walk_tau_careful(const DepositArgs &a, const PairInput &in, int S,
                                              unsigned long long *lo, unsigned long long *hi,
                                              int *bad, int lane, Counters &ct)
{
    Tau64 s;
    if (!s.setup(a.lp, in))
        return;
    Counters c{};
    walk_tau<0, COUNT, 1>(a, s, S, lo, hi, bad, lane, nullptr, c);
    if (COUNT) {
        ct.c += c.a + c.b + c.c;
        ct.pixels += c.pixels;
    }
}

// ------------------------------------------------------ far-field tiles
// Far in a pair's damping wing (every pixel of a tile beyond the multipole
// radius and at least TILE_DIST pixels from the line centre) the FP32 form
// does not deposit pixel by pixel.  The bins are cut into tiles of TILE_W
// pixels; for a tile that lies wholly inside the pair's window, the pair adds
// its contribution at TILE_M Chebyshev nodes of the tile to per-tile node
// accumulators (the same split fixed point as the pixels).  When the sightline
// is complete each pixel adds the polynomial interpolant of its tile's node
// sums, which is linear in the node values and so equals the sum over pairs of
// each pair's interpolant.  The far wing is a polynomial in 1/V^2 (pole at
// V = 0), so with the tile half-width at most 0.2 of the distance to the pole
// the interpolation error of 8 Chebyshev nodes is below 5e-7 of the value
// (1/V^2: 2.3e-7, 1/V^4: 6.2e-6 times its share, at most a few percent that
// far out; 10 nodes gave 3e-9 for 2.7% more deposit time).
// The window rule needs no per-pixel test inside such a tile: the far wing
// decreases with |V| (STAGE_TILES), and its value equals tautail at a radius
// V_stop found once per pair by Newton's method on the multipole polynomial;
// a tile whose farthest pixel centre lies within 0.999 V_stop has every pixel
// above tautail by far more than the FP32 rounding (the wing falls as 1/V^2,
// so 2e-3 of tautail), and the window continues past it.  The tile holding the
// stop pixel, a tile cut by the wrap of the bins and the nbins/2 cap are
// walked pixel by pixel as before.  The (tile, node) items of a run of tiles
// are spread over the 32 lanes.
constexpr int TILE_W = 64;
constexpr int TILE_M = 8;
constexpr float TILE_DIST = 128.f;

__device__ double g_tile_w[TILE_W * TILE_M];   // [pixel in tile][node] interpolation weights
__device__ float g_tile_x[TILE_M];             // node positions, pixels from the tile's first

// Node positions x_k = 31.5 (1 + cos((2k+1) pi / 2M)) rounded to float, and
// the barycentric Lagrange weights of those float positions at the pixels.
__global__ void tile_weights_kernel()
{
    const int t = threadIdx.x;
    if (t >= TILE_W * TILE_M)
        return;
    const int p = t / TILE_M, k = t % TILE_M;
    const double h = 0.5 * (TILE_W - 1);
    double x[TILE_M];
#pragma unroll
    for (int i = 0; i < TILE_M; i++)
        x[i] = (double)(float)(h + h * cos((2 * i + 1) * PI_D / (2 * TILE_M)));
    double num = 0.0, den = 0.0;
    bool hit = false;
#pragma unroll
    for (int i = 0; i < TILE_M; i++) {
        double lam = 1.0;
#pragma unroll
        for (int j = 0; j < TILE_M; j++)
            if (j != i)
                lam /= (x[i] - x[j]);
        const double d = (double)p - x[i];
        if (d == 0.0) {
            hit = true;
            num = (i == k) ? 1.0 : 0.0;
            break;
        }
        den += lam / d;
        if (i == k)
            num = lam / d;
    }
    g_tile_w[t] = hit ? num : num / den;
    if (p == 0)
        g_tile_x[k] = (float)x[k];
}

// |V| (in units of b) where the far wing equals tautail: the root of
// h(W) = sum_r A_r W^(r+1) = tautail in W = 1/V^2.  h is increasing and convex
// for A_r >= 0, so Newton's method from W0 = tautail / A_0 (h(W0) >= tautail)
// decreases monotonically to the root.  Returns +inf when tautail <= 0 (the
// window then runs to the cap) and 0 when the wing is identically zero.
__device__ __forceinline__ float far_stop_radius(const Tau32 &s, float tautail)
{
    if (!(tautail > 0.f))
        return __int_as_float(0x7f800000);
    if (!(s.A[0] > 0.f))
        return 0.f;
    float W = tautail / s.A[0];
#pragma unroll 1
    for (int it = 0; it < 4; it++) {
        float h = s.A[MP_R - 1], d = (float)MP_R * s.A[MP_R - 1];
#pragma unroll
        for (int r = MP_R - 2; r >= 0; r--) {
            h = fmaf(h, W, s.A[r]);
            d = fmaf(d, W, (float)(r + 1) * s.A[r]);
        }
        W -= (h * W - tautail) / d;
    }
    return W > 0.f ? rsqrtf(W) : __int_as_float(0x7f800000);
}

// The FP32 walk of one pair (not the counting variant; with tlo null, or a
// pair without STAGE_TILES, it is walk_tau's pixel walk).  Pixel steps as in
// walk_tau; once the walk is far (see above) a step ends at the next tile
// boundary, and at a boundary the run of sure tiles ahead is deposited through
// its nodes, 32 (tile, node) items per round.  Pixel steps and node rounds
// share one evaluation per lane per iteration.
__device__ __forceinline__ void walk_tau32_tiled(const DepositArgs &a, const Tau32 &s, int S,
                                                 unsigned long long *lo, unsigned long long *hi,
                                                 unsigned long long *tlo,
                                                 unsigned long long *thi, int *bad, int lane,
                                                 const float2 *tab)
{
    const int nbins = a.lp.nbins;
    const int half = nbins / 2;
    const float tautail = (float)a.lp.tautail;
    const int j0 = s.j0;
    const float lane_f = (float)lane;
    const float dmin = fmaxf(s.vmp, TILE_DIST * s.vk);
    float vsure = -1.f;
    for (int dir = 0; dir < 2; dir++) {
        bool far = false, tiles = s.tiles && tlo != nullptr;
        int k = 0;
        int n = 0, items = 0, base = 0, jb_run = 0;   // node run state
        while (k < half) {
            const int koff0 = dir == 0 ? k : -1 - k;
            const float kf0 = (float)koff0;
            int len = 32;
            if (items == 0 && tiles) {
                if (!far) {
                    const float ve = dir == 0 ? fmaf(kf0, s.vk, s.v0) : -fmaf(kf0 + 1.f, s.vk, s.v0);
                    far = ve >= dmin;
                }
                if (far) {
                    const int jb = bin_from(j0, koff0, nbins);
                    const int rem = dir == 0 ? (TILE_W - jb % TILE_W) % TILE_W
                                             : (jb + 1) % TILE_W;
                    if (rem == 0) {
                        if (vsure < 0.f)
                            vsure = 0.999f * far_stop_radius(s, tautail);
                        const float klim = dir == 0 ? (vsure - s.vmid0) / s.vk
                                                    : (vsure + s.vmid0) / s.vk - 1.f;
                        n = 0;
                        if (klim >= (float)k + (float)(TILE_W - 1))
                            n = (int)fminf((klim - (float)k + 1.f) / (float)TILE_W, 1e6f);
                        n = min(n, (half - k) / TILE_W);
                        n = min(n, dir == 0 ? (nbins - jb) / TILE_W : (jb + 1) / TILE_W);
                        if (n > 0) {
                            items = n * TILE_M;
                            base = 0;
                            jb_run = jb;
                        } else {
                            tiles = dir == 0 ? (nbins - jb < TILE_W) : false;
                        }
                    } else {
                        len = min(32, rem);
                    }
                }
            }
            // one evaluation per lane: a tile node (node rounds) or a pixel
            float ka, kb;
            int idx = 0;
            bool on = false;
            if (items) {
                const int it0 = base + lane;
                on = it0 < items;
                const int it = on ? it0 : 0;
                const int t = it / TILE_M, m = it - t * TILE_M;
                const int kt = k + TILE_W * t;
                ka = (float)(dir == 0 ? kt : -kt - TILE_W);
                kb = g_tile_x[m];
                idx = (dir == 0 ? jb_run + TILE_W * t : jb_run - TILE_W * (t + 1) + 1) / TILE_W *
                          TILE_M + m;
            } else {
                ka = dir == 0 ? kf0 + lane_f : kf0 - lane_f;
                kb = 0.f;
            }
            const float v = s.value_at(ka, kb, tab);
            if (items) {
                if (on)
                    accumulate<float, 1>(a.dev_err, v, idx, S, tlo, thi, bad);
                base += 32;
                if (base >= items) {
                    k += TILE_W * n;
                    items = 0;
                }
                continue;
            }
            const int kk = k + lane;
            const bool valid = lane < len && kk < half;
            const bool stop = valid && (v < tautail);
            const unsigned msk = __ballot_sync(0xffffffffu, stop);
            const int last = msk ? (__ffs(msk) - 1) : 31;
            if (valid && lane <= last)
                accumulate<float, 1>(a.dev_err, v, bin_from(j0, dir == 0 ? kk : -1 - kk, nbins),
                                     S, lo, hi, bad);
            if (msk)
                break;
            k += len;
        }
    }
}

// FP32 tau form: the warps of the CTA take chunks of `chunk` consecutive pairs
// of the sightline from a shared counter (dynamic balance: pair costs differ by
// orders of magnitude); each lane sets up one pair of the chunk into the warp's
// staging area, then the warp walks the chunk's pairs one after another.
template <bool COUNT, bool REC>
__device__ __forceinline__ void deposit_pairs32(const DepositArgs &a, int axis, long long e0,
                                                long long e1, int S, unsigned long long *lo,
                                                unsigned long long *hi, unsigned long long *tlo,
                                                unsigned long long *thi, int *bad,
                                                Stage32 *sw, unsigned *s_chunk,
                                                const float2 *vtab, double bintov_d, int lane,
                                                Counters &ct)
{
    const int chunk = a.chunk;
    const float bintov_f = (float)bintov_d;
    const Setup32 k32(a.lp, bintov_d);
    for (;;) {
        unsigned c = 0;
        if (lane == 0)
            c = atomicAdd(s_chunk, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        const long long cb = e0 + (long long)c * chunk;
        if (cb >= e1)
            break;
        const int n = (int)min((long long)chunk, e1 - cb);
        const PairRec *rec = REC ? reinterpret_cast<const PairRec *>(a.pl.rec) : nullptr;
        if constexpr (REC) {
            const int w = threadIdx.x >> 5;
            unsigned long long *mbar = &s_stage_bar[w];
            const unsigned mphase = s_stage_phase[w];
            // the chunk's records land in the warp's staging area (n x 32 bytes:
            // 16-byte aligned at both ends, within the chunk x 80-byte area)
            PairRec *rb = reinterpret_cast<PairRec *>(sw);
            fence_proxy_async_shared();   // earlier reads of the area come first
            __syncwarp();
            if (lane == 0)
                bulk_copy_g2s(rb, rec + cb, (unsigned)n * (unsigned)sizeof(PairRec), mbar);
            bool landed = mbar_wait(mbar, mphase, STAGE_WAIT_TRIES);
            if (!landed) {
                if (lane == 0)
                    atomicOr(a.dev_err, (unsigned)DEVERR_STAGE_WAIT);
                landed = mbar_wait(mbar, mphase, STAGE_WAIT_TRIES);
            }
            PairRec r{};
            if (lane < n && landed)
                r = rb[lane];
            __syncwarp();
            if (lane == 0)
                s_stage_phase[w] = mphase ^ 1u;
            if (lane < n) {
                Stage32 st;
                if (!landed || !stage32_setup(a.lp, k32, rec_input(r), bintov_d, st, nullptr))
                    st.flags = STAGE_SKIP;
                sw[lane] = st;
            }
        } else if (lane < n) {
            const PairInput in = load_pair(a.p, a.pl, cb + lane, axis, true, a.dev_err);
            Stage32 st;
            if (!stage32_setup(a.lp, k32, in, bintov_d, st, nullptr))
                st.flags = STAGE_SKIP;
            sw[lane] = st;
        }
        (void)rec;
        __syncwarp();
        for (int k = 0; k < n; k++) {
            const Stage32 st = sw[k];
            if (st.flags & STAGE_SKIP)
                continue;
            if (st.flags & STAGE_CAREFUL) {
                const PairInput in = REC ? rec_input(rec[cb + k])
                                         : load_pair(a.p, a.pl, cb + k, axis, true, a.dev_err);
                walk_tau_careful<COUNT>(a, in, S, lo, hi, bad, lane, ct);
                continue;
            }
            Tau32 s;
            s.load(st, bintov_f);
            if constexpr (!COUNT)
                walk_tau32_tiled(a, s, S, lo, hi, tlo, thi, bad, lane, vtab);
            else
                walk_tau<1, COUNT, 1>(a, s, S, lo, hi, bad, lane, vtab, ct);
        }
        __syncwarp();
    }
}

// FP32 column density: chunks of staged pairs as in deposit_pairs32.
template <bool COUNT>
__device__ __forceinline__ void deposit_pairs_col32(const DepositArgs &a, int axis,
                                                    long long e0, long long e1, int S,
                                                    unsigned long long *lo,
                                                    unsigned long long *hi, int *bad,
                                                    StageCol32 *sw, unsigned *s_chunk,
                                                    double btk, int lane, Counters &ct)
{
    const int chunk = a.chunk, nbins = a.lp.nbins, kernel = a.lp.kernel;
    const float box_f = (float)btk;
    for (;;) {
        unsigned c = 0;
        if (lane == 0)
            c = atomicAdd(s_chunk, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        const long long cb = e0 + (long long)c * chunk;
        if (cb >= e1)
            break;
        const int n = (int)min((long long)chunk, e1 - cb);
        if (lane < n) {
            const PairInput in = load_pair(a.p, a.pl, cb + lane, axis, false, a.dev_err);
            StageCol32 st;
            stagecol32_setup(a.lp, in, btk, st);
            sw[lane] = st;
        }
        __syncwarp();
        for (int q = 0; q < n; q++) {
            const StageCol32 st = sw[q];
            if (st.flags == COL_SKIP)
                continue;
            if (st.flags == COL_BAD) {
                if (lane == 0)
                    atomicOr(a.dev_err, (unsigned)DEVERR_WINDOW_LIMIT);
                *bad = 1;
                continue;
            }
            int j = st.j0 + lane;
            while (j >= nbins)
                j -= nbins;
            for (int k = lane; k <= st.kmax; k += 32) {
                float v;
                if (k == 0)
                    v = st.e0;
                else if (k == st.kmax)
                    v = st.e2;
                else if (k == st.kmax - 1)
                    v = st.e1;
                else
                    v = colden_interior32(st, kernel, box_f, k);
                accumulate<float, 1>(a.dev_err, v, j, S, lo, hi, bad);
                if (COUNT)
                    ct.pixels++;
                j += 32;
                while (j >= nbins)
                    j -= nbins;
            }
        }
        __syncwarp();
    }
}

// MAXT: the block size the kernel is compiled for (launch bound).  The FP32
// optical-depth deposit has 512-, 768- and 1024-thread builds (128, 80 and 64
// registers per thread: 16, 24 or 32 warps per SM with the sightline's
// accumulators on chip); the autotuner picks among them.
// REC: the FP32 optical-depth deposit through pair records (PairRec; the
// buffer is a.pl.rec) instead of gathering from the particle arrays.
template <bool TAU, int PREC, bool COUNT, int MAXT = (PREC == 0 ? 256 : 512), bool REC = false>
__global__ void __launch_bounds__(MAXT, 1)
    deposit_kernel(DepositArgs a)
{
    extern __shared__ __align__(16) unsigned long long smem[];
    __shared__ BoundScratch red;
    __shared__ float2 vtab[FSG_V32_N];
    __shared__ int s_bad;
    __shared__ unsigned s_ticket, s_chunk;
    const int nbins = a.lp.nbins;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    PairRec *rec = nullptr;
    if constexpr (REC) {
        static_assert(TAU && PREC == 1 && !COUNT, "records serve the FP32 optical depth");
        rec = reinterpret_cast<PairRec *>(a.pl.rec);
        if (lane == 0) {
            mbar_init(&s_stage_bar[warp], 1);
            s_stage_phase[warp] = 0u;
        }
        __syncthreads();
    }
    const double boxtokpc = a.lp.vbox / nbins / a.lp.velfac;
    const double bintov_d = a.lp.vbox / nbins;
    Counters ct{};
    if constexpr (PREC == 1 && TAU)
        stage_voigt32(vtab);
    const Bound32 bk(a.lp);
    // dynamic shared memory: [accumulators lo, hi (smem_mode)] [pair staging]
    // [far-field tile nodes lo, hi (tiles)]
    Stage32 *stage = reinterpret_cast<Stage32 *>(smem + (a.smem_mode ? 2 * (size_t)nbins : 0));
    StageCol32 *stage_col = reinterpret_cast<StageCol32 *>(stage);
    const int ntiles = nbins / TILE_W;
    const int nnodes = ntiles * TILE_M;
    unsigned long long *tlo = nullptr, *thi = nullptr;
    if (TAU && PREC == 1 && !COUNT && a.tiles && a.smem_mode) {
        tlo = reinterpret_cast<unsigned long long *>(stage + nwarps * a.chunk);
        thi = tlo + nnodes;
    }
    const float btk_abs = (float)fabs(boxtokpc);
    const float col_kfac = (float)(kernel_max(a.lp.kernel) * 1.001);

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
        const auto bf = [&](long long e) {
            const PairInput in = load_pair(a.p, a.pl, e, axis, TAU, a.dev_err);
            if constexpr (REC) {
                rec[e] = make_rec(in, a.pl.part[e]);   // for the second pass and the staging
                return tau_pair_bound32(bk, in);
            } else if constexpr (TAU && PREC == 1)
                return tau_pair_bound32(bk, in);
            else if constexpr (!TAU && PREC == 1)
                return colden_pair_bound32(a.lp, in, btk_abs, col_kfac);
            else
                return TAU ? tau_pair_bound(a.lp, in) : colden_pair_bound(a.lp, in, boxtokpc);
        };
        double B;
        if constexpr (REC) {
            B = order_free_bound(e0, e1, bf, [&](long long e) {
                return tau_pair_bound32(bk, rec_input(rec[e]));
            }, &red);
            // the records are read by bulk copies (async proxy) after the barrier below
            fence_proxy_async_global();
        } else {
            B = order_free_bound(e0, e1, bf, bf, &red);
        }
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
        if (tlo)
            for (int j = threadIdx.x; j < nnodes; j += blockDim.x) {
                tlo[j] = 0ull;
                thi[j] = 0ull;
            }
        if (threadIdx.x == 0)
            s_chunk = 0u;
        __syncthreads();
        const int S = (B > 0.0 && !s_bad) ? (PREC == 0 ? 124 : SPLIT_TOP) - ilogb(B) : 0;
        // 2. deposit: warp per pair
        if constexpr (TAU && PREC == 1) {
            if (!s_bad && B > 0.0)
                deposit_pairs32<COUNT, REC>(a, axis, e0, e1, S, lo, hi, tlo, thi, &s_bad,
                                       stage + warp * a.chunk, &s_chunk, vtab, bintov_d, lane,
                                       ct);
        } else if constexpr (!TAU && PREC == 1) {
            if (!s_bad && B > 0.0)
                deposit_pairs_col32<COUNT>(a, axis, e0, e1, S, lo, hi, &s_bad,
                                           stage_col + warp * a.chunk, &s_chunk, boxtokpc, lane,
                                           ct);
        } else if (!s_bad && B > 0.0) {
            for (long long e = e0 + warp; e < e1; e += nwarps) {
                const PairInput in = load_pair(a.p, a.pl, e, axis, TAU, a.dev_err);
                if constexpr (TAU) {
                    Tau64 s;
                    if (s.setup(a.lp, in))
                        walk_tau<0, COUNT, 0>(a, s, S, lo, hi, &s_bad, lane, vtab, ct);
                } else {
                    Colden c;
                    if (c.setup(a.lp, in, boxtokpc)) {
                        if (!c.ok) {
                            if (lane == 0)
                                atomicOr(a.dev_err, (unsigned)DEVERR_WINDOW_LIMIT);
                            s_bad = 1;
                        } else {
                            walk_colden<PREC, COUNT>(a, c, S, lo, hi, &s_bad, lane, ct);
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
            if (tlo) {
                // node sums to double in place, then pixel + its tile's interpolant
                double *node = reinterpret_cast<double *>(tlo);
                for (int j = threadIdx.x; j < nnodes; j += blockDim.x)
                    node[j] = from_split(tlo[j], thi[j], S);
                __syncthreads();
                for (int j = threadIdx.x; j < nbins; j += blockDim.x) {
                    double v = from_split(lo[j], hi[j], S);
                    if (j < ntiles * TILE_W) {
                        const double *w = g_tile_w + (j % TILE_W) * TILE_M;
                        const double *nd = node + (j / TILE_W) * TILE_M;
                        double f = 0.0;
#pragma unroll
                        for (int m = 0; m < TILE_M; m++)
                            f = fma(w[m], nd[m], f);
                        v += f;
                    }
                    row[j] = v;
                }
            } else {
                for (int j = threadIdx.x; j < nbins; j += blockDim.x)
                    row[j] = PREC == 0 ? from_fixed(lo[j], hi[j], S) : from_split(lo[j], hi[j], S);
            }
        }
        if (!a.persistent)
            break;
        __syncthreads();
        if (threadIdx.x == 0)
            s_ticket = atomicAdd(a.ticket, 1u);
        __syncthreads();
        ticket = s_ticket;
    }
    if constexpr (COUNT) {
        atomicAdd(&a.counters[0], ct.a);
        atomicAdd(&a.counters[1], ct.b);
        atomicAdd(&a.counters[2], ct.c);
        atomicAdd(&a.counters[3], ct.pixels);
        atomicAdd(&a.counters[4], ct.d);
        atomicAdd(&a.counters[5], ct.e);
        atomicAdd(&a.counters[6], ct.f);
        atomicAdd(&a.counters[7], ct.g);
    }
}

// Fallback for sightlines with non-finite contributions: FP64 atomics straight
// into the output row, so inf and NaN combine as the reference's += does.
template <bool TAU>
__global__ void __launch_bounds__(256) fallback_kernel(LineParams lp, LineTables t, Particles p,
                                                       PairLists pl, const int *bad_lines,
                                                       const int *n_bad_dev, double *out,
                                                       unsigned *dev_err)
{
    // with n_bad_dev the grid covers every sightline and the count is read here
    if (n_bad_dev && (int)blockIdx.x >= *n_bad_dev)
        return;
    const int line = bad_lines[blockIdx.x];
    const int axis = t.axis[line];
    const int nbins = lp.nbins;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const double boxtokpc = lp.vbox / nbins / lp.velfac;
    double *row = out + (size_t)line * nbins;
    const long long e0 = pl.off[line], e1 = pl.off[line + 1];
    Counters ct{};
    for (long long e = e0 + warp; e < e1; e += nwarps) {
        const PairInput in = load_pair(p, pl, e, axis, TAU, dev_err);
        if (TAU) {
            Tau64 s;
            if (!s.setup(lp, in))
                continue;
            const int half = nbins / 2;
            const int j0 = wrap_bin(s.zmax, nbins);
            for (int dir = 0; dir < 2; dir++) {
                for (int step = 0; step < half; step += 32) {
                    const int k = step + lane;
                    const bool valid = k < half;
                    const int koff = dir == 0 ? k : -1 - k;
                    double tl = 0.0;
                    if (valid)
                        tl = s.taulast<false>(koff, dev_err, ct);
                    const unsigned m = __ballot_sync(0xffffffffu, valid && tl < lp.tautail);
                    const int last = m ? (__ffs(m) - 1) : 31;
                    if (valid && lane <= last)
                        atomicAdd(&row[bin_from(j0, koff, nbins)], tl);
                    if (m)
                        break;
                }
            }
        } else {
            Colden c;
            if (!c.setup(lp, in, boxtokpc))
                continue;
            if (!c.ok) {
                if (lane == 0)
                    atomicOr(dev_err, (unsigned)DEVERR_WINDOW_LIMIT);
                continue;
            }
            for (long long z = c.zlow + lane; z <= c.zhigh; z += 32)
                atomicAdd(&row[wrap_bin(z, nbins)], c.value64(z));
        }
    }
}

// ============================================================ column density, K channels
// K weighted column densities of one sightline set in one pass (the weighted
// compute_tau=0 calls of Spectra.get_velocity / get_temp /
// get_dens_weighted_density, spectra.py:945-1043, differ only in the density
// array).  Each pixel's kernel integral is computed once and multiplied by
// each channel's density; per channel the bound, the fixed-point scale, the
// rounding of every contribution and the integer sums are those of a
// single-channel deposit, so every channel equals its single-channel result
// bit for bit.
struct ChannelArgs {
    LineParams lp;
    LineTables t;
    Particles p;             // dens unused
    PairLists pl;
    const int *line_order;
    int nlos;
    int nch;
    const float *dens[MAX_CHANNELS];
    double *out[MAX_CHANNELS];
    int *bad_lines;          // [nch][nlos]
    int *n_bad;              // [nch]
    unsigned *ticket;
    unsigned *dev_err;
    unsigned long long *gacc;   // per-CTA accumulators when not in shared memory
    int smem_mode;
    int chunk;
};

// Staged pair of the FP32 multi-channel form (96 bytes): the geometry of
// StageCol32 with the three FP64 edge integrals kept density-free in double.
struct __align__(16) StageColK {
    int j0, kmax, flags, pad;
    double kf0, kf1, kf2;    // kern_frac of pixels 0, kmax - 1, kmax
    float dL0, dR0, two_zr, inv_h2, ch, pad1;
    float dens[MAX_CHANNELS];
};
static_assert(sizeof(StageColK) == 96, "StageColK is six 16-byte words");

__device__ __forceinline__ PairInput load_pair_ch(const ChannelArgs &a, long long e, int axis,
                                                  int c)
{
    Particles p = a.p;
    p.dens = a.dens[c];
    return load_pair(p, a.pl, e, axis, false, a.dev_err);
}

template <int PREC>
__global__ void __launch_bounds__(PREC == 0 ? 256 : 512) colden_channels_kernel(ChannelArgs a)
{
    extern __shared__ __align__(16) unsigned long long smem[];
    __shared__ BoundScratch red;
    __shared__ int s_bad[MAX_CHANNELS];
    __shared__ double s_B[MAX_CHANNELS];
    __shared__ unsigned s_ticket, s_chunk;
    const int nbins = a.lp.nbins, nch = a.nch;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double btk = a.lp.vbox / nbins / a.lp.velfac;
    const float btk_abs = (float)fabs(btk);
    const float col_kfac = (float)(kernel_max(a.lp.kernel) * 1.001);
    const size_t acc_words = 2 * (size_t)nbins * nch;
    unsigned long long *acc = a.smem_mode ? smem : a.gacc + (size_t)blockIdx.x * acc_words;
    StageColK *sw = reinterpret_cast<StageColK *>(smem + (a.smem_mode ? acc_words : 0)) +
                    warp * a.chunk;
    if (threadIdx.x == 0)
        s_ticket = atomicAdd(a.ticket, 1u);
    __syncthreads();
    unsigned ticket = s_ticket;
    while (ticket < (unsigned)a.nlos) {
        const int line = a.line_order[ticket];
        const int axis = a.t.axis[line];
        const long long e0 = a.pl.off[line], e1 = a.pl.off[line + 1];
        // 1. per-channel bounds, summed exactly as the single-channel deposit sums them
        for (int c = 0; c < nch; c++) {
            const auto bf = [&](long long e) {
                const PairInput in = load_pair_ch(a, e, axis, c);
                return PREC == 1 ? colden_pair_bound32(a.lp, in, btk_abs, col_kfac)
                                 : colden_pair_bound(a.lp, in, btk);
            };
            const double B = order_free_bound(e0, e1, bf, bf, &red);
            if (threadIdx.x == 0) {
                s_B[c] = B;
                s_bad[c] = !isfinite(B);
            }
        }
        for (size_t j = threadIdx.x; j < acc_words; j += blockDim.x)
            acc[j] = 0ull;
        if (threadIdx.x == 0)
            s_chunk = 0u;
        __syncthreads();
        int S[MAX_CHANNELS];
        bool live[MAX_CHANNELS];
#pragma unroll
        for (int c = 0; c < MAX_CHANNELS; c++) {
            live[c] = c < nch && !s_bad[c] && s_B[c] > 0.0;
            S[c] = live[c] ? (PREC == 0 ? 124 : SPLIT_TOP) - ilogb(s_B[c]) : 0;
        }
        // 2. deposit: chunks of pairs, one lane per pair of the chunk sets it up
        for (;;) {
            unsigned q = 0;
            if (lane == 0)
                q = atomicAdd(&s_chunk, 1u);
            q = __shfl_sync(0xffffffffu, q, 0);
            const long long cb = e0 + (long long)q * a.chunk;
            if (cb >= e1)
                break;
            const int n = (int)min((long long)a.chunk, e1 - cb);
            if (lane < n) {
                const PairInput in = load_pair_ch(a, cb + lane, axis, 0);
                StageColK st;
                Colden col;
                st.flags = 0;
                if (!col.setup(a.lp, in, btk)) {
                    st.flags = COL_SKIP;
                } else if (!col.ok) {
                    st.flags = COL_BAD;
                } else {
                    st.j0 = wrap_bin(col.zlow, nbins);
                    st.kmax = (int)col.kmax;
                    const auto kf = [&](long long z) {
                        const double plow = __dsub_rn(__dmul_rn(btk, (double)z), col.pos1);
                        return kern_frac<double>(a.lp.kernel, plow, __dadd_rn(plow, btk), col.smooth,
                                                 col.dr2, col.zrange);
                    };
                    if constexpr (PREC == 1) {
                        st.kf0 = kf(col.zlow);
                        st.kf1 = col.kmax >= 2 ? kf(col.zlow + col.kmax - 1) : 0.0;
                        st.kf2 = col.kmax >= 1 ? kf(col.zhigh) : 0.0;
                        st.dL0 = col.dL0;
                        st.dR0 = col.dR0;
                        st.two_zr = col.two_zr;
                        st.inv_h2 = col.inv_h2;
                        st.ch = col.ch;
                    }
                }
                const int ip = a.pl.part[cb + lane];
#pragma unroll
                for (int c = 0; c < MAX_CHANNELS; c++)
                    st.dens[c] = (c < nch && (unsigned long long)(long long)ip <
                                                 (unsigned long long)a.p.n)
                                     ? __ldg(&a.dens[c][ip]) : 0.f;
                sw[lane] = st;
            }
            __syncwarp();
            for (int k2 = 0; k2 < n; k2++) {
                const StageColK st = sw[k2];
                if (st.flags == COL_SKIP)
                    continue;
                if (st.flags == COL_BAD) {
                    if (lane == 0)
                        atomicOr(a.dev_err, (unsigned)DEVERR_WINDOW_LIMIT);
                    for (int c = 0; c < nch; c++)
                        s_bad[c] = 1;
                    continue;
                }
                // the FP64 form needs the pair's geometry again: rebuild it from the pair
                Colden col;
                if constexpr (PREC == 0) {
                    const PairInput in = load_pair_ch(a, cb + k2, axis, 0);
                    col.setup(a.lp, in, btk);
                }
                int j = st.j0 + lane;
                while (j >= nbins)
                    j -= nbins;
                for (int k = lane; k <= st.kmax; k += 32) {
                    if constexpr (PREC == 0) {
                        const double plow = __dsub_rn(__dmul_rn(btk, (double)(col.zlow + k)),
                                                      col.pos1);
                        const double f = kern_frac<double>(a.lp.kernel, plow, __dadd_rn(plow, btk),
                                                           col.smooth, col.dr2, col.zrange);
#pragma unroll
                        for (int c = 0; c < MAX_CHANNELS; c++)
                            if (live[c])
                                accumulate<double, 0>(a.dev_err, (double)st.dens[c] * f, j, S[c],
                                                      acc + 2 * (size_t)c * nbins,
                                                      acc + (2 * (size_t)c + 1) * nbins,
                                                      &s_bad[c]);
                    } else {
                        const bool edge = k == 0 || k >= st.kmax - 1;
                        const double fe = k == 0 ? st.kf0 : (k == st.kmax ? st.kf2 : st.kf1);
                        float f32 = 0.f;
                        if (!edge) {
                            StageCol32 g;
                            g.kmax = st.kmax;
                            g.dens_f = 1.f;
                            g.dL0 = st.dL0;
                            g.dR0 = st.dR0;
                            g.two_zr = st.two_zr;
                            g.inv_h2 = st.inv_h2;
                            g.ch = st.ch;
                            // unit density: the single-channel form multiplies this by dens
                            f32 = colden_interior32(g, a.lp.kernel, (float)btk, k);
                        }
#pragma unroll
                        for (int c = 0; c < MAX_CHANNELS; c++)
                            if (live[c]) {
                                const float v = edge ? (float)((double)st.dens[c] * fe)
                                                     : st.dens[c] * f32;
                                accumulate<float, 1>(a.dev_err, v, j, S[c],
                                                     acc + 2 * (size_t)c * nbins,
                                                     acc + (2 * (size_t)c + 1) * nbins,
                                                     &s_bad[c]);
                            }
                    }
                    j += 32;
                    while (j >= nbins)
                        j -= nbins;
                }
            }
            __syncwarp();
        }
        __syncthreads();
        // 3. flush each channel's row (or hand the line to the fallback)
        for (int c = 0; c < nch; c++) {
            if (s_bad[c]) {
                if (threadIdx.x == 0)
                    a.bad_lines[(size_t)c * a.nlos + atomicAdd(&a.n_bad[c], 1)] = line;
            } else if (s_B[c] > 0.0) {
                double *row = a.out[c] + (size_t)line * nbins;
                const unsigned long long *lo = acc + 2 * (size_t)c * nbins, *hi = lo + nbins;
                for (int j = threadIdx.x; j < nbins; j += blockDim.x)
                    row[j] = PREC == 0 ? from_fixed(lo[j], hi[j], S[c])
                                       : from_split(lo[j], hi[j], S[c]);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0)
            s_ticket = atomicAdd(a.ticket, 1u);
        __syncthreads();
        ticket = s_ticket;
    }
}

// ============================================================ backward
// dL/d(dens), dL/dT and dL/d(v_los) per particle from dL/dtau per pixel, for
// the FP32 form.  The window of every pair is recomputed with the forward's
// stop rule (and is treated as fixed, like the sub-sample count).  For a pair
// with tau contribution c_j = scale * S_j, S_j = sum_i w_i H(u_ij, a):
//   dc_j/d(dens)  = scale_nod * S_j
//   dc_j/d(v_los) = scale / b * sum_i w_i dH/du          (du/dv = 1/b)
//   dc_j/dT       = -scale / (2T) * sum_i w_i (H + u dH/du + a dH/da)
// (amp ~ 1/b, u ~ 1/b, a ~ 1/b and db/dT = b/(2T)).
struct GradArgs {
    LineParams lp;
    LineTables t;
    Particles p;
    PairLists pl;
    const int *line_order;
    int nlos;
    const double *grad_tau;
    float *g_dens, *g_temp, *g_vel;
    unsigned *ticket;
    unsigned *dev_err;
};

struct GradSums {
    float d, v, t;
};

__device__ __forceinline__ GradSums grad_node_sums(const Tau32 &s, float V, const float2 *tab)
{
    GradSums g = {0.f, 0.f, 0.f};
    // the small-damping form when every node of every lane is inside its table
    // (max_i |U_i - V| = |V| + |U_6|; uniform over the warp)
    const bool small =
        s.vc.a <= VOIGT_SMALL_A &&
        __all_sync(0xffffffffu, fabsf(V) + fabsf(s.U[NODES - 1]) < VOIGT_SMALL_X);
    if (small) {
#pragma unroll
        for (int i = 0; i < NODES; ++i) {
            const float u = s.U[i] - V;
            const VoigtGrad r = voigt_grad_small32(u, s.vc);
            g.d = fmaf(s.w[i], r.h, g.d);
            g.v = fmaf(s.w[i], r.hu, g.v);
            g.t = fmaf(s.w[i], r.h + fmaf(u, r.hu, s.aa_f * r.ha), g.t);
        }
        return g;
    }
#pragma unroll
    for (int i = 0; i < NODES; ++i) {
        const float u = s.U[i] - V;
        const VoigtGrad r = voigt_grad32(u, s.vc, tab);
        g.d = fmaf(s.w[i], r.h, g.d);
        g.v = fmaf(s.w[i], r.hu, g.v);
        g.t = fmaf(s.w[i], r.h + fmaf(u, r.hu, s.aa_f * r.ha), g.t);
    }
    return g;
}

// FP64 profile and central-difference derivatives for the rare pairs that the
// FP32 form walks in FP64 (Tau32::careful).
__device__ __noinline__ void voigt_grad64(double u, double a, double &h, double &hu, double &ha)
{
    h = voigt_f64(u, a);
    const double eu = 1e-6 * fmax(1.0, fabs(u));
    hu = (voigt_f64(u + eu, a) - voigt_f64(u - eu, a)) / (2.0 * eu);
    const double ea = 1e-6 * fmax(fabs(a), 1e-8);
    ha = (voigt_f64(u, a + ea) - voigt_f64(u, a - ea)) / (2.0 * ea);
}

__device__ __noinline__ void grad_pair_careful(const GradArgs &a, const PairInput &in,
                                               const double *gt, int lane, double &gd,
                                               double &gv, double &gtmp)
{
    Tau64 s;
    gd = gv = gtmp = 0.0;
    if (!s.setup(a.lp, in))
        return;
    const int nbins = a.lp.nbins, half = nbins / 2;
    const int j0 = wrap_bin(s.zmax, nbins);
    const double amp_v = s.ampd / a.lp.velfac;   // amp dens / velfac
    const double amp_nod = (s.ampd / ((double)in.dens != 0.0 ? (double)in.dens : 1.0)) /
                           a.lp.velfac;
    Counters ct{};
    for (int dir = 0; dir < 2; dir++) {
        for (int step = 0; step < half; step += 32) {
            const int k = step + lane;
            const bool valid = k < half;
            const int koff = dir == 0 ? k : -1 - k;
            double tl = 0.0, sd = 0.0, sv = 0.0, stt = 0.0;
            if (valid) {
                tl = s.taulast<false>(koff, a.dev_err, ct);
                const double vlow = (double)(s.zmax + koff) * s.bintov - s.vel;
                const double vhigh = vlow + s.bintov;
                int np = 1;
                double dv = 0.0;
                if (!((vhigh - vlow) < s.half_b)) {
                    const double npd = 2 * ceil((vhigh - vlow) / s.half_b / 2) + 1.;
                    np = npd <= MAX_SUBSAMPLES ? (int)npd : 1;
                    dv = (vhigh - vlow) / (np - 1);
                }
                for (int q = 0; q < np; q++) {
                    const double vo = np == 1 ? (vhigh + vlow) / 2. : vlow + q * dv;
                    const double wq = (np == 1) ? 1.0 : ((q == 0 || q == np - 1) ? 0.5 : 1.0) /
                                                           (np - 1);
                    for (int i = 0; i < NODES; ++i) {
                        const double u = (s.vv[i] - vo) * s.inv_b;
                        double h, hu, ha;
                        voigt_grad64(u, s.aa, h, hu, ha);
                        const double ww = wq * s.w[i] * s.deltav;
                        sd += ww * h;
                        sv += ww * hu;
                        stt += ww * (h + u * hu + s.aa * ha);
                    }
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, valid && tl < a.lp.tautail);
            const int last = m ? (__ffs(m) - 1) : 31;
            if (valid && lane <= last) {
                const double g = gt[bin_from(j0, koff, nbins)];
                gd += g * amp_nod * sd;
                gv += g * amp_v * s.inv_b * sv;
                gtmp += g * (-amp_v / (2.0 * (double)in.temp)) * stt;
            }
            if (m)
                break;
        }
    }
}

// Staged pair of the backward kernel: the forward constants plus what the
// gradient needs (96 bytes).
struct __align__(16) StageGrad {
    Stage32 s;
    float scale_nod, temp;
    int ip, pad;
};
// 1024 threads at 64 registers (32 warps per SM; the kernel spills the same
// ~250 bytes at 128 registers), 16 staged pairs per warp.
constexpr int GRAD_THREADS = 1024, GRAD_CHUNK = 16;
constexpr size_t GRAD_SMEM = (size_t)(GRAD_THREADS / 32) * GRAD_CHUNK * sizeof(StageGrad);

// One warp, one FP32-walk pair: dL/d(dens), dL/d(v_los), dL/dT summed over the
// pair's window (all lanes hold the sums afterwards).
__device__ __forceinline__ void grad_pair32(const Tau32 &s, const double *gt, int nbins,
                                            float tautail, int lane, const float2 *vtab,
                                            float &ad, float &av, float &at)
{
    const int half = nbins / 2;
    const int j0 = s.j0;
    const float lane_f = (float)lane;
    ad = av = at = 0.f;
    for (int dir = 0; dir < 2; dir++) {
        float kf = dir == 0 ? lane_f : -1.0f - lane_f;
        const float dkf = dir == 0 ? 32.0f : -32.0f;
        for (int step = 0; step < half; step += 32, kf += dkf) {
            const int k = step + lane;
            const bool valid = k < half;
            const int koff = dir == 0 ? k : -1 - k;
            const float vlow_b = fmaf(kf, s.bintov, s.base0) * s.inv_b;
            GradSums g;
            if (s.npoints == 1) {
                g = grad_node_sums(s, vlow_b + s.hbin_b, vtab);
            } else {
                g = grad_node_sums(s, vlow_b, vtab);
                g.d *= 0.5f;
                g.v *= 0.5f;
                g.t *= 0.5f;
                for (int i = 1; i < s.npoints - 1; ++i) {
                    const GradSums h = grad_node_sums(s, fmaf((float)i, s.sub_dv, vlow_b), vtab);
                    g.d += h.d;
                    g.v += h.v;
                    g.t += h.t;
                }
                const GradSums h = grad_node_sums(s, vlow_b + 2.f * s.hbin_b, vtab);
                g.d += 0.5f * h.d;
                g.v += 0.5f * h.v;
                g.t += 0.5f * h.t;
            }
            const float tl = s.scale * g.d;
            const unsigned m = __ballot_sync(0xffffffffu, valid && tl < tautail);
            const int last = m ? (__ffs(m) - 1) : 31;
            if (valid && lane <= last) {
                const float gg = (float)gt[bin_from(j0, koff, nbins)];
                ad = fmaf(gg, g.d, ad);
                av = fmaf(gg, g.v, av);
                at = fmaf(gg, g.t, at);
            }
            if (m)
                break;
        }
    }
}

// Sightlines from a ticket queue; within a sightline the warps take chunks of
// pairs from a shared counter, each lane sets up one pair of the chunk (the
// forward's lane-parallel setup) and the warp walks them one after another.
__global__ void __launch_bounds__(GRAD_THREADS, 1) grad_kernel(GradArgs a)
{
    extern __shared__ __align__(16) unsigned char gsmem[];
    __shared__ float2 vtab[FSG_V32_N];
    __shared__ unsigned s_ticket, s_chunk;
    stage_voigt32(vtab);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nbins = a.lp.nbins;
    const float tautail = (float)a.lp.tautail;
    const double bintov_d = a.lp.vbox / nbins;
    const float bintov_f = (float)bintov_d;
    const Setup32 k32(a.lp, bintov_d);
    StageGrad *sw = reinterpret_cast<StageGrad *>(gsmem) + warp * GRAD_CHUNK;
    if (threadIdx.x == 0)
        s_ticket = atomicAdd(a.ticket, 1u);
    __syncthreads();
    unsigned ticket = s_ticket;
    while (ticket < (unsigned)a.nlos) {
        const int line = a.line_order[ticket];
        const int axis = a.t.axis[line];
        const double *gt = a.grad_tau + (size_t)line * nbins;
        const long long e0 = a.pl.off[line], e1 = a.pl.off[line + 1];
        if (threadIdx.x == 0)
            s_chunk = 0u;
        __syncthreads();
        for (;;) {
            unsigned c = 0;
            if (lane == 0)
                c = atomicAdd(&s_chunk, 1u);
            c = __shfl_sync(0xffffffffu, c, 0);
            const long long cb = e0 + (long long)c * GRAD_CHUNK;
            if (cb >= e1)
                break;
            const int n = (int)min((long long)GRAD_CHUNK, e1 - cb);
            if (lane < n) {
                const PairInput in = load_pair(a.p, a.pl, cb + lane, axis, true, a.dev_err);
                StageGrad g;
                g.temp = in.temp;
                g.ip = a.pl.part[cb + lane];
                g.pad = 0;
                if (!stage32_setup(a.lp, k32, in, bintov_d, g.s, &g.scale_nod))
                    g.s.flags = STAGE_SKIP;
                sw[lane] = g;
            }
            __syncwarp();
            for (int k = 0; k < n; k++) {
                const StageGrad g = sw[k];
                if (g.s.flags & STAGE_SKIP)
                    continue;
                float gd = 0.f, gv = 0.f, gtmp = 0.f;
                if (g.s.flags & STAGE_CAREFUL) {
                    const PairInput in = load_pair(a.p, a.pl, cb + k, axis, true, a.dev_err);
                    double d_, v_, t_;
                    grad_pair_careful(a, in, gt, lane, d_, v_, t_);
                    gd = (float)d_;
                    gv = (float)v_;
                    gtmp = (float)t_;
                } else {
                    Tau32 s;
                    s.load(g.s, bintov_f);
                    float ad, av, at;
                    grad_pair32(s, gt, nbins, tautail, lane, vtab, ad, av, at);
                    gd = g.scale_nod * ad;
                    gv = s.scale * s.inv_b * av;
                    gtmp = -s.scale / (2.0f * g.temp) * at;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    gd += __shfl_xor_sync(0xffffffffu, gd, o);
                    gv += __shfl_xor_sync(0xffffffffu, gv, o);
                    gtmp += __shfl_xor_sync(0xffffffffu, gtmp, o);
                }
                if (lane == 0) {
                    atomicAdd(&a.g_dens[g.ip], gd);
                    atomicAdd(&a.g_temp[g.ip], gtmp);
                    atomicAdd(&a.g_vel[3ll * g.ip + axis - 1], gv);
                }
            }
            __syncwarp();
        }
        __syncthreads();
        if (threadIdx.x == 0)
            s_ticket = atomicAdd(a.ticket, 1u);
        __syncthreads();
        ticket = s_ticket;
    }
}

int g_max_smem_optin = -1;

// The kernel build for a block size: the FP32 tau form (not counting) has
// 768- and 1024-thread builds beside the default.
// The kernel build for a block size and input path: the FP32 optical-depth
// deposit has 512-, 768- and 1024-thread builds, each gathering the particle
// fields or reading pair records.
template <bool TAU, int PREC, bool COUNT>
decltype(&deposit_kernel<TAU, PREC, COUNT>) deposit_build(int threads, bool rec)
{
    if constexpr (TAU && PREC == 1 && !COUNT) {
        if (rec) {
            if (threads > 768)
                return deposit_kernel<TAU, PREC, COUNT, 1024, true>;
            if (threads > 512)
                return deposit_kernel<TAU, PREC, COUNT, 768, true>;
            return deposit_kernel<TAU, PREC, COUNT, 512, true>;
        }
        if (threads > 768)
            return deposit_kernel<TAU, PREC, COUNT, 1024, false>;
        if (threads > 512)
            return deposit_kernel<TAU, PREC, COUNT, 768, false>;
    }
    (void)rec;
    return deposit_kernel<TAU, PREC, COUNT>;
}

template <bool TAU, int PREC, bool COUNT>
void launch_one(const DepositArgs &a, int grid, int threads, size_t smem, cudaStream_t s)
{
    auto k = deposit_build<TAU, PREC, COUNT>(threads, a.pl.rec != nullptr);   // launcher: cfg.rec
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<grid, threads, smem, s>>>(a);
}

template <bool TAU, int PREC, bool COUNT>
int resident_ctas(int threads, size_t smem, bool rec)
{
    auto k = deposit_build<TAU, PREC, COUNT>(threads, rec);
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, threads, smem);
    return n;
}

}  // namespace

namespace {
int max_smem_optin()
{
    if (g_max_smem_optin < 0) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        g_max_smem_optin = v;
    }
    return g_max_smem_optin;
}
// static shared memory of the deposit kernel is < 1.5 KiB
constexpr int STATIC_SMEM_RESERVE = 2048;
}  // namespace

namespace {
size_t stage_pair_bytes(int compute_tau, int precision)
{
    if (precision != 1)
        return 0;
    return compute_tau ? sizeof(Stage32) : sizeof(StageCol32);
}
}  // namespace

size_t deposit_smem_bytes(const DepositLaunch &cfg, int compute_tau, int nbins)
{
    return (cfg.smem_mode ? (size_t)16 * nbins : 0) +
           (size_t)(cfg.threads / 32) * cfg.chunk * stage_pair_bytes(compute_tau, cfg.precision) +
           (cfg.tiles ? (size_t)16 * TILE_M * (nbins / TILE_W) : 0);
}

void deposit_plan(DepositLaunch &cfg, int compute_tau, int nbins)
{
    const size_t cap = (size_t)(max_smem_optin() - STATIC_SMEM_RESERVE);
    if (cfg.precision == 1) {
        // staged pairs per warp (cfg.chunk > 0: as requested): by default 8 for
        // tau (finer chunks balance the warps better at the end of a
        // sightline, where pair costs differ most), 32 (or 16 to keep the
        // accumulators on chip) for the column density; far-field tiles (tau)
        // when their node accumulators fit beside the pixel accumulators,
        // unless switched off
        const int first = compute_tau ? 8 : 32;
        const int asked = cfg.chunk;
        const bool want_tiles = compute_tau && cfg.tiles;
        for (int tiles : {1, 0}) {
            if (tiles && !want_tiles)
                continue;
            cfg.tiles = tiles;
            for (int chunk : {first, 16, 8}) {
                if (asked > 0)
                    chunk = asked;
                else if (chunk > first)
                    continue;
                cfg.chunk = chunk;
                cfg.smem_mode = 1;
                if (deposit_smem_bytes(cfg, compute_tau, nbins) <= cap)
                    return;
                if (asked > 0)
                    break;
            }
        }
        cfg.tiles = 0;
        cfg.chunk = asked > 0 ? asked : first;
        cfg.smem_mode = 0;
        return;
    }
    cfg.chunk = 0;
    cfg.tiles = 0;
    cfg.smem_mode = (size_t)16 * nbins <= cap;
}

int deposit_max_smem_bins(int compute_tau, int precision, int threads)
{
    const size_t stage = (size_t)(threads / 32) * 8 * stage_pair_bytes(compute_tau, precision);
    return (int)(((size_t)(max_smem_optin() - STATIC_SMEM_RESERVE) - stage) / 16);
}

int deposit_resident_ctas(const DepositLaunch &cfg, int compute_tau, int nbins)
{
    const size_t smem = deposit_smem_bytes(cfg, compute_tau, nbins);
    const int threads = cfg.threads;
    if (compute_tau)
        return cfg.precision ? resident_ctas<true, 1, false>(threads, smem, cfg.rec != 0)
                             : resident_ctas<true, 0, false>(threads, smem, false);
    return cfg.precision ? resident_ctas<false, 1, false>(threads, smem, false)
                         : resident_ctas<false, 0, false>(threads, smem, false);
}

int launch_deposit(const LineParams &lp, const LineTables &t, const Particles &p,
                   const PairLists &pl, const int *line_order, int nlos, double *out,
                   unsigned *ticket, int *bad_lines, int *n_bad, unsigned *dev_err,
                   unsigned long long *gacc, unsigned long long *counters,
                   const DepositLaunch &cfg, cudaStream_t s)
{
    if (nlos == 0)
        return 0;
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
    a.counters = counters;
    a.smem_mode = cfg.smem_mode;
    a.persistent = cfg.persistent;
    a.chunk = cfg.chunk;
    a.tiles = cfg.tiles;
    // records only for the launch that asked for them (the buffer may be shared)
    if (!(cfg.rec && cfg.precision == 1 && lp.compute_tau && counters == nullptr))
        a.pl.rec = nullptr;
    const size_t smem = deposit_smem_bytes(cfg, lp.compute_tau, lp.nbins);
    int launched = 1;
    if (cfg.tiles && counters == nullptr) {
        tile_weights_kernel<<<1, TILE_W * TILE_M, 0, s>>>();
        launched++;
    }
    const int grid = cfg.persistent ? cfg.grid : nlos;
    const int threads = cfg.threads;
    const bool count = counters != nullptr;
    if (lp.compute_tau) {
        if (cfg.precision == 0)
            count ? launch_one<true, 0, true>(a, grid, threads, smem, s)
                  : launch_one<true, 0, false>(a, grid, threads, smem, s);
        else
            count ? launch_one<true, 1, true>(a, grid, threads, smem, s)
                  : launch_one<true, 1, false>(a, grid, threads, smem, s);
    } else {
        if (cfg.precision == 0)
            count ? launch_one<false, 0, true>(a, grid, threads, smem, s)
                  : launch_one<false, 0, false>(a, grid, threads, smem, s);
        else
            count ? launch_one<false, 1, true>(a, grid, threads, smem, s)
                  : launch_one<false, 1, false>(a, grid, threads, smem, s);
    }
    return launched;
}

void launch_deposit_fallback(const LineParams &lp, const LineTables &t, const Particles &p,
                             const PairLists &pl, const int *bad_lines, int n_bad, double *out,
                             unsigned *dev_err, cudaStream_t s)
{
    if (n_bad <= 0)
        return;
    if (lp.compute_tau)
        fallback_kernel<true><<<n_bad, 256, 0, s>>>(lp, t, p, pl, bad_lines, nullptr, out,
                                                    dev_err);
    else
        fallback_kernel<false><<<n_bad, 256, 0, s>>>(lp, t, p, pl, bad_lines, nullptr, out,
                                                     dev_err);
}

void launch_deposit_fallback_dev(const LineParams &lp, const LineTables &t, const Particles &p,
                                 const PairLists &pl, const int *bad_lines, const int *n_bad_dev,
                                 int nlos, double *out, unsigned *dev_err, cudaStream_t s)
{
    if (nlos <= 0)
        return;
    if (lp.compute_tau)
        fallback_kernel<true><<<nlos, 256, 0, s>>>(lp, t, p, pl, bad_lines, n_bad_dev, out,
                                                   dev_err);
    else
        fallback_kernel<false><<<nlos, 256, 0, s>>>(lp, t, p, pl, bad_lines, n_bad_dev, out,
                                                    dev_err);
}

void launch_tau_backward(const LineParams &lp, const LineTables &t, const Particles &p,
                         const PairLists &pl, const int *line_order, int nlos,
                         const double *grad_tau, float *g_dens, float *g_temp, float *g_vel,
                         unsigned *ticket, unsigned *dev_err, int grid, cudaStream_t s)
{
    if (nlos == 0 || lp.nbins == 0)
        return;
    GradArgs a;
    a.lp = lp;
    a.t = t;
    a.p = p;
    a.pl = pl;
    a.line_order = line_order;
    a.nlos = nlos;
    a.grad_tau = grad_tau;
    a.g_dens = g_dens;
    a.g_temp = g_temp;
    a.g_vel = g_vel;
    a.ticket = ticket;
    a.dev_err = dev_err;
    cudaFuncSetAttribute(grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)GRAD_SMEM);
    grad_kernel<<<grid, GRAD_THREADS, GRAD_SMEM, s>>>(a);
}

int tau_backward_resident_ctas()
{
    int n = 0;
    cudaFuncSetAttribute(grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)GRAD_SMEM);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, grad_kernel, GRAD_THREADS, GRAD_SMEM);
    return n;
}


// ---------------------------------------------------------------- K channels
namespace {
constexpr int CHAN_CHUNK = 32;
int chan_threads(int precision) { return precision == 0 ? 256 : 512; }
size_t chan_smem(int precision, int nch, int nbins, int smem_mode)
{
    return (smem_mode ? 2 * sizeof(unsigned long long) * nbins * nch : 0) +
           (size_t)(chan_threads(precision) / 32) * CHAN_CHUNK * sizeof(StageColK);
}
template <int PREC>
void chan_attr(size_t smem)
{
    cudaFuncSetAttribute(colden_channels_kernel<PREC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
}
}  // namespace

ChannelPlan colden_channels_plan(int precision, int nch, int nbins)
{
    ChannelPlan pl{};
    pl.threads = chan_threads(precision);
    const size_t cap = (size_t)(max_smem_optin() - STATIC_SMEM_RESERVE);
    pl.smem_mode = chan_smem(precision, nch, nbins, 1) <= cap;
    pl.smem = chan_smem(precision, nch, nbins, pl.smem_mode);
    int n = 0;
    if (precision == 0) {
        chan_attr<0>(pl.smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, colden_channels_kernel<0>, pl.threads,
                                                      pl.smem);
    } else {
        chan_attr<1>(pl.smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, colden_channels_kernel<1>, pl.threads,
                                                      pl.smem);
    }
    pl.per_sm = n > 0 ? n : 1;
    pl.acc_words_per_cta = 2 * (size_t)nbins * nch;
    return pl;
}

void launch_colden_channels(const LineParams &lp, const LineTables &t, const Particles &p,
                            const PairLists &pl, const int *line_order, int nlos, int nch,
                            const float *const *dens, double *const *out, int *bad_lines,
                            int *n_bad, unsigned *ticket, unsigned *dev_err,
                            unsigned long long *gacc, int precision, const ChannelPlan &plan,
                            int grid, cudaStream_t s)
{
    if (nlos == 0 || nch == 0)
        return;
    ChannelArgs a;
    a.lp = lp;
    a.t = t;
    a.p = p;
    a.pl = pl;
    a.line_order = line_order;
    a.nlos = nlos;
    a.nch = nch;
    for (int c = 0; c < MAX_CHANNELS; c++) {
        a.dens[c] = c < nch ? dens[c] : nullptr;
        a.out[c] = c < nch ? out[c] : nullptr;
    }
    a.bad_lines = bad_lines;
    a.n_bad = n_bad;
    a.ticket = ticket;
    a.dev_err = dev_err;
    a.gacc = gacc;
    a.smem_mode = plan.smem_mode;
    a.chunk = CHAN_CHUNK;
    if (precision == 0) {
        chan_attr<0>(plan.smem);
        colden_channels_kernel<0><<<grid, plan.threads, plan.smem, s>>>(a);
    } else {
        chan_attr<1>(plan.smem);
        colden_channels_kernel<1><<<grid, plan.threads, plan.smem, s>>>(a);
    }
}

}  // namespace fsg

