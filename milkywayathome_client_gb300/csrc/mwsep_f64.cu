/* mwsep_f64.cu -- plain FP64 integral and likelihood kernels (the drop-in
 * form, MWSEP_PLAIN_F64).
 *
 * Arithmetic: FP64 throughout (mwsep_f64_point.cuh): the likelihood in the
 * reference's own operation order (convolve_f64), the integral in the
 * completed-square form (convolve_f64_cs), compiled with -fmad=false.  Per
 * cell the convolution points are summed in order n = 0..C-1, then
 * multiplied by reff_xr_rp3 and by the cell volume V = irv[k]*ids[j]
 * (cpu/evaluation_optimized.c:500-504, :513).  Cells are Kahan-summed per
 * thread, then combined error-free across the block; blocks are combined by
 * mwsep_reduce.cu in a fixed order.
 *
 * Mapping: one thread owns a (mu, nu) column and a contiguous run of
 * k_chunk r-bins ("item", mwsep::item_pos); consecutive threads own
 * consecutive columns of the same r-run, so every r-bin table read is
 * warp-uniform.  Grid-stride loop over the items of the cells the area
 * integrates (all of them, or a rank's slice); gridDim.y indexes the
 * parameter vector of a batch.
 */
#include <cuda_runtime.h>
#include <math.h>
#include "mwsep_internal.h"
#include "mwsep_reduce.cuh"
#include "mwsep_f64_point.cuh"

namespace {

using namespace mwsep::f64;
using mwsep::comp_sum;

template <int SMAX>
__global__ void __launch_bounds__(256) integral_f64_kernel(const mwsep_area_dev A,
                                                           const mwsep_theta_consts* __restrict__ thetas,
                                                           double2* __restrict__ partials,
                                                           long long theta_stride)
{
    __shared__ mwsep_theta_consts th;
    __shared__ double red[2 * (1 + SMAX) * 32];
    __shared__ double etab[kExpTable];
    load_theta(th, thetas + blockIdx.y);
    exp_tang_table(etab);
    __syncthreads();

    comp_sum acc[1 + SMAX];
#pragma unroll
    for (int k = 0; k < 1 + SMAX; ++k) acc[k].zero();

    const int S = th.n_streams;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x; item < A.n_items; item += stride)
        integral_item<SMAX>(A, th, etab, item, acc);
    mwsep::block_reduce<1 + SMAX>(acc, red);
    if (threadIdx.x == 0)
    {
        double2* out = partials + (size_t)blockIdx.y * theta_stride + (size_t)blockIdx.x * (1 + S);
        out[0] = make_double2(acc[0].s, acc[0].c);
#pragma unroll
        for (int s = 0; s < SMAX; ++s)
            if (s < S) out[1 + s] = make_double2(acc[1 + s].s, acc[1 + s].c);
    }
}

/* calculate_likelihood per star (cpu/evaluation_optimized.c:665-717).
 * integrals: [theta][1+S] after the cut subtraction.
 * Partial slots: [0] sum log10 p, [1] zero count, [2] bg-only sum,
 * [3+s] stream-only sums. */
template <int SMAX>
__global__ void __launch_bounds__(256) likelihood_f64_kernel(const mwsep_stars_dev St,
                                                             const mwsep_theta_consts* __restrict__ thetas,
                                                             const double* __restrict__ integrals,
                                                             double2* __restrict__ partials,
                                                             long long theta_stride)
{
    __shared__ mwsep_theta_consts th;
    __shared__ double red[2 * (3 + SMAX) * 32];
    load_theta(th, thetas + blockIdx.y);
    __syncthreads();
    const int S = th.n_streams;
    const double* I = integrals + (size_t)blockIdx.y * (1 + S);

    comp_sum acc[3 + SMAX];
#pragma unroll
    for (int k = 0; k < 3 + SMAX; ++k) acc[k].zero();

    const int N = St.n_stars;
    for (int s0 = blockIdx.x * blockDim.x + threadIdx.x; s0 < N; s0 += gridDim.x * blockDim.x)
        likelihood_star<SMAX>(St, th, I, s0, acc);
    mwsep::block_reduce<3 + SMAX>(acc, red);
    if (threadIdx.x == 0)
    {
        double2* out = partials + (size_t)blockIdx.y * theta_stride + (size_t)blockIdx.x * (3 + S);
#pragma unroll
        for (int k = 0; k < 3 + SMAX; ++k)
            if (k < 3 + S) out[k] = make_double2(acc[k].s, acc[k].c);
    }
}

template <int SMAX>
int launch_integral(const mwsep_area_dev* A, const mwsep_theta_consts* th, const mwsep_launch_shape* sh,
                    double2* partials, cudaStream_t st)
{
    const long long ncomp = 1 + sh->n_streams;
    const long long theta_stride = (long long)sh->n_areas * sh->grid * ncomp;
    dim3 g(sh->grid, sh->n_theta);
    integral_f64_kernel<SMAX><<<g, sh->block, 0, st>>>(*A, th, partials + (size_t)sh->area_index * sh->grid * ncomp,
                                                        theta_stride);
    return (int)cudaGetLastError();
}

template <int SMAX>
int launch_likelihood(const mwsep_stars_dev* S, const mwsep_theta_consts* th, const mwsep_launch_shape* sh,
                      const double* integrals, double2* partials, cudaStream_t st)
{
    const long long theta_stride = (long long)sh->grid * (3 + sh->n_streams);
    dim3 g(sh->grid, sh->n_theta);
    likelihood_f64_kernel<SMAX><<<g, sh->block, 0, st>>>(*S, th, integrals, partials, theta_stride);
    return (int)cudaGetLastError();
}

} // namespace

extern "C" int mwsep_integral_f64_blocks_per_sm(int n_streams, int block)
{
    int b = 0;
    cudaError_t e;
    if (n_streams <= 1) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, integral_f64_kernel<1>, block, 0);
    else if (n_streams <= 2) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, integral_f64_kernel<2>, block, 0);
    else if (n_streams <= 4) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, integral_f64_kernel<4>, block, 0);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, integral_f64_kernel<8>, block, 0);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return 1;
    }
    return b > 0 ? b : 1;
}

extern "C" int mwsep_launch_integral_f64(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                                         const mwsep_launch_shape* sh, double2* partials, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (sh->n_streams <= 1) return launch_integral<1>(area, th_dev, sh, partials, st);
    if (sh->n_streams <= 2) return launch_integral<2>(area, th_dev, sh, partials, st);
    if (sh->n_streams <= 4) return launch_integral<4>(area, th_dev, sh, partials, st);
    return launch_integral<8>(area, th_dev, sh, partials, st);
}

extern "C" int mwsep_launch_likelihood_f64(const mwsep_stars_dev* stars, const mwsep_theta_consts* th_dev,
                                           const mwsep_launch_shape* sh, const double* integrals,
                                           double2* partials, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (sh->n_streams <= 1) return launch_likelihood<1>(stars, th_dev, sh, integrals, partials, st);
    if (sh->n_streams <= 2) return launch_likelihood<2>(stars, th_dev, sh, integrals, partials, st);
    if (sh->n_streams <= 4) return launch_likelihood<4>(stars, th_dev, sh, integrals, partials, st);
    return launch_likelihood<8>(stars, th_dev, sh, integrals, partials, st);
}

MWSEP_CHECKS_READER(mwsep_checks_f64)
