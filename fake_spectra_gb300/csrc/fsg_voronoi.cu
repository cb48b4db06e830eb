// Voronoi-mesh sightline cells (kernel 2): the GPU form of
// IndexTable::assign_cells (fake_spectra/index_table.cpp:152-223).
//
// A sightline is sampled at N = int(box / 0.1) points x_i = (i + 1/2) box/N.
// Each point belongs to the nearest of the sightline's particles (periodic
// 3-D distance in double, the first in ascending particle order on a tie, as
// the reference's strict '<' over its std::map gives).  The reference walks
// the points in order; the cell of point 0 may wrap around the box, and the
// walk stops at the first point past box/2 that belongs to it again.  Here:
//   1. the cell of point 0 (first_cell_kernel),
//   2. the stop point: the first such point past box/2 (wrap_point_kernel),
//   3. first/last/count of the points of every cell before the stop point
//      (cell_extent_kernel),
//   4. each cell's float segment [left, right], rounded as the reference's
//      float array is, with the contiguity the reference asserts checked by
//      the count (cell_segment_kernel).
// The nearest-cell search takes the cells in shared-memory tiles: an FP32
// distance prefilter, then the reference's double distance on the cells
// within the float error bound of the float minimum.
#include "fsg_internal.cuh"

namespace fsg {

namespace {

constexpr double RESO = 0.1;   // index_table.h:8
constexpr int VOR_THREADS = 256;
constexpr int VOR_TILE = 1024;

struct VorArgs {
    const float *pos;          // [3N]
    const int *part;           // pairs, ascending particle order within a sightline
    const long long *off;      // [L+1]
    const int *axis;           // [L]
    const double *cofm;        // [3L]
    int nlos, npoint;
    double box, reso;
};

__device__ __forceinline__ double min_image(double d, double box)
{
    d = fabs(d);
    return d > box / 2. ? box - d : d;
}

__device__ __forceinline__ float min_image_f(float d, float box)
{
    d = fabsf(d);
    return d > 0.5f * box ? box - d : d;
}

// Cell (index within the sightline's list) nearest to point x of line l; the
// whole block calls it with its own points (x < 0: the thread has none).
__device__ int nearest_cell(const VorArgs &a, int l, double x, float3 *tile)
{
    const long long e0 = a.off[l];
    const int m = (int)(a.off[l + 1] - e0);
    const int ax = a.axis[l];
    const int i1 = ax % 3, i2 = (ax + 1) % 3;
    const double yp = a.cofm[3 * (size_t)l + i1], zp = a.cofm[3 * (size_t)l + i2];
    const float boxf = (float)a.box, xf = (float)x, ypf = (float)yp, zpf = (float)zp;
    // pass 1: float minimum
    float best_f = 3.4e38f;
    for (int t0 = 0; t0 < m; t0 += VOR_TILE) {
        const int tn = min(VOR_TILE, m - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < tn; k += blockDim.x) {
            const float *p = &a.pos[3 * (size_t)a.part[e0 + t0 + k]];
            tile[k] = make_float3(p[ax - 1], p[i1], p[i2]);
        }
        __syncthreads();
        if (x >= 0.0)
            for (int k = 0; k < tn; k++) {
                const float3 q = tile[k];
                const float dx = min_image_f(q.x - xf, boxf), dy = min_image_f(q.y - ypf, boxf),
                            dz = min_image_f(q.z - zpf, boxf);
                best_f = fminf(best_f, sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))));
            }
    }
    // pass 2: the reference's double distance on the candidates, in order
    const float margin = 1e-6f * boxf + 1e-5f * best_f;
    double best = a.box;
    int best_k = 0;
    for (int t0 = 0; t0 < m; t0 += VOR_TILE) {
        const int tn = min(VOR_TILE, m - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < tn; k += blockDim.x) {
            const float *p = &a.pos[3 * (size_t)a.part[e0 + t0 + k]];
            tile[k] = make_float3(p[ax - 1], p[i1], p[i2]);
        }
        __syncthreads();
        if (x >= 0.0)
            for (int k = 0; k < tn; k++) {
                const float3 q = tile[k];
                const float dx = min_image_f(q.x - xf, boxf), dy = min_image_f(q.y - ypf, boxf),
                            dz = min_image_f(q.z - zpf, boxf);
                if (sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) > best_f + margin)
                    continue;
                const double ddx = min_image((double)q.x - x, a.box);
                const double ddy = min_image((double)q.y - yp, a.box);
                const double ddz = min_image((double)q.z - zp, a.box);
                const double d = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx),
                                                                __dmul_rn(ddy, ddy)),
                                                      __dmul_rn(ddz, ddz)));
                if (d < best) {
                    best = d;
                    best_k = t0 + k;
                }
            }
    }
    return best_k;
}

__device__ __forceinline__ double point_x(const VorArgs &a, int i) { return (i + 0.5) * a.reso; }

__global__ void __launch_bounds__(VOR_THREADS) first_cell_kernel(VorArgs a, int line0, int *c0)
{
    __shared__ float3 tile[VOR_TILE];
    const int l = line0 + blockIdx.y;
    if (a.off[l + 1] == a.off[l])
        return;
    const int k = nearest_cell(a, l, threadIdx.x == 0 ? point_x(a, 0) : -1.0, tile);
    if (threadIdx.x == 0)
        c0[l] = k;
}

__global__ void __launch_bounds__(VOR_THREADS) wrap_point_kernel(VorArgs a, int line0,
                                                                 const int *c0, int *istar)
{
    __shared__ float3 tile[VOR_TILE];
    const int l = line0 + blockIdx.y;
    if (a.off[l + 1] == a.off[l])
        return;
    const int i = blockIdx.x * VOR_THREADS + threadIdx.x;
    const double x = point_x(a, i);
    const bool mine = i < a.npoint && x > a.box / 2. + 0.5 * a.reso;
    const int k = nearest_cell(a, l, mine ? x : -1.0, tile);
    if (mine && k == c0[l])
        atomicMin(&istar[l], i);
}

__global__ void __launch_bounds__(VOR_THREADS) cell_extent_kernel(VorArgs a, int line0,
                                                                  const int *istar, int *first,
                                                                  int *last, int *cnt)
{
    __shared__ float3 tile[VOR_TILE];
    const int l = line0 + blockIdx.y;
    const long long e0 = a.off[l];
    if (a.off[l + 1] == e0)
        return;
    const int i = blockIdx.x * VOR_THREADS + threadIdx.x;
    const bool mine = i < a.npoint && i < istar[l];
    const int k = nearest_cell(a, l, mine ? point_x(a, i) : -1.0, tile);
    if (mine) {
        atomicMin(&first[e0 + k], i);
        atomicMax(&last[e0 + k], i);
        atomicAdd(&cnt[e0 + k], 1);
    }
}

// One thread per pair: the float segment of its cell.
__global__ void cell_segment_kernel(VorArgs a, const int *c0, const int *istar,
                                    const int *first, const int *last, const int *cnt,
                                    const int *pair_line, float2 *seg, unsigned *dev_err,
                                    long long npairs)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= npairs)
        return;
    const int l = pair_line[e];
    const int k = (int)(e - a.off[l]);
    float left, right;
    if (cnt[e] == 0) {
        left = right = (float)(3 * a.box);
    } else {
        if (cnt[e] != last[e] - first[e] + 1)
            atomicOr(dev_err, (unsigned)DEVERR_VORONOI_CELL);   // the reference exits here
        left = (float)point_x(a, first[e]);
        right = (float)point_x(a, last[e]);
    }
    if (k == c0[l] && istar[l] < a.npoint) {   // the first cell wraps around the box
        left = (float)point_x(a, istar[l]);
        right = (float)((double)right + a.box);
    }
    seg[e] = make_float2((float)((double)left - 0.5 * a.reso), (float)((double)right + 0.5 * a.reso));
}

__global__ void pair_line_kernel(const long long *off, int nlos, int *pair_line)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nlos)
        return;
    for (long long e = off[l]; e < off[l + 1]; e++)
        pair_line[e] = l;
}

__global__ void fill_int_kernel(int *p, long long n, int v)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        p[i] = v;
}

unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

long long voronoi_scratch_ints(long long npairs, int nlos)
{
    return 4 * npairs + 2 * (long long)nlos;
}

void launch_voronoi_cells(const float *pos, const int *part, const long long *off,
                          const int *axis, const double *cofm, int nlos, long long npairs,
                          double box, int *scratch, float2 *seg, unsigned *dev_err,
                          cudaStream_t s)
{
    if (nlos <= 0 || npairs <= 0)
        return;
    VorArgs a;
    a.pos = pos;
    a.part = part;
    a.off = off;
    a.axis = axis;
    a.cofm = cofm;
    a.nlos = nlos;
    a.npoint = (int)(box / RESO);
    a.box = box;
    a.reso = box / a.npoint;
    int *first = scratch, *last = first + npairs, *cnt = last + npairs, *pline = cnt + npairs;
    int *c0 = pline + npairs, *istar = c0 + nlos;
    fill_int_kernel<<<blocks_for(npairs, 256), 256, 0, s>>>(first, npairs, 0x7fffffff);
    fill_int_kernel<<<blocks_for(npairs, 256), 256, 0, s>>>(last, npairs, -1);
    fill_int_kernel<<<blocks_for(npairs, 256), 256, 0, s>>>(cnt, npairs, 0);
    fill_int_kernel<<<blocks_for(nlos, 256), 256, 0, s>>>(c0, nlos, 0);
    fill_int_kernel<<<blocks_for(nlos, 256), 256, 0, s>>>(istar, nlos, a.npoint);
    pair_line_kernel<<<blocks_for(nlos, 256), 256, 0, s>>>(off, nlos, pline);
    const unsigned px = blocks_for(a.npoint, VOR_THREADS);
    for (int l0 = 0; l0 < nlos; l0 += 65535) {
        const unsigned ny = (unsigned)std::min(65535, nlos - l0);
        first_cell_kernel<<<dim3(1, ny), VOR_THREADS, 0, s>>>(a, l0, c0);
        wrap_point_kernel<<<dim3(px, ny), VOR_THREADS, 0, s>>>(a, l0, c0, istar);
        cell_extent_kernel<<<dim3(px, ny), VOR_THREADS, 0, s>>>(a, l0, istar, first, last, cnt);
    }
    cell_segment_kernel<<<blocks_for(npairs, 256), 256, 0, s>>>(a, c0, istar, first, last, cnt,
                                                                pline, seg, dev_err, npairs);
}

}  // namespace fsg
