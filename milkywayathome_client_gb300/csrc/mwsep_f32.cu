/* mwsep_f32.cu -- compensated-FP32 integral and likelihood kernels
 * (MWSEP_MIXED_F32) for one evaluation or a batch of parameter vectors on
 * one resident wedge.  The density arithmetic is in mwsep_f32_point.cuh.
 *
 * Kernels are specialised on the exact stream count (0..4; 8 covers 5..8
 * with guards) and on the background form, so the inner loop carries no
 * dead work.
 */
#include <cuda_runtime.h>
#include <math.h>
#include "milkyway_separation_gb300_test.h"
#include "mwsep_internal.h"
#include "mwsep_reduce.cuh"
#include "mwsep_f32_point.cuh"

namespace {

using namespace mwsep::f32;

constexpr int kBlock = 256;
#ifndef MWSEP_F32_MINB
#define MWSEP_F32_MINB 2 /* 2 x 256 threads per SM: <= 128 registers, no spills up to 3 streams */
#endif

template <int S, int FORM>
__global__ void __launch_bounds__(kBlock, MWSEP_F32_MINB) integral_f32_kernel(const mwsep_area_dev A,
                                                                 const mwsep_theta_consts* __restrict__ thetas,
                                                                 double2* __restrict__ partials,
                                                                 long long theta_stride)
{
    __shared__ mwsep_theta_consts th;
    __shared__ double red[2 * (1 + S) * 32];
    load_theta(th, thetas + blockIdx.y);
    __syncthreads();
    /* a batch mixing background forms gets one launch per form */
    if (mwsep_bg_form(&th) != FORM) return;

    double acc[1 + S];
#pragma unroll
    for (int k = 0; k < 1 + S; ++k) acc[k] = 0.0;

    const BgConsts bc = bg_consts(th);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x; item < A.n_items; item += stride)
        integral_item<S, FORM>(A, th, bc, item, acc);
    reduce_and_store<1 + S>(acc, 1 + th.n_streams, red,
                            partials + (size_t)blockIdx.y * theta_stride + (size_t)blockIdx.x * (1 + th.n_streams));
}

/* The same integral over warp tiles (A.warp_items == 1): each warp takes
 * tiles wt = warp, warp + warps, ... of the grid. */
template <int S, int FORM>
__global__ void __launch_bounds__(kBlock, MWSEP_F32_MINB) integral_f32w_kernel(const mwsep_area_dev A,
                                                                  const mwsep_theta_consts* __restrict__ thetas,
                                                                  double2* __restrict__ partials,
                                                                  long long theta_stride)
{
    __shared__ mwsep_theta_consts th;
    __shared__ ThetaDF<S> td;
    __shared__ double red[2 * (1 + S) * 32];
    __shared__ __align__(16) float cs[kBlock / 32][TileSmem<S>::N];
    load_theta(th, thetas + blockIdx.y);
    __syncthreads();
    if (mwsep_bg_form(&th) != FORM) return;
    theta_df_part<S>(th, td, (int)threadIdx.x);
    __syncthreads();

    double acc[1 + S];
#pragma unroll
    for (int k = 0; k < 1 + S; ++k) acc[k] = 0.0;

    const BgConsts bc = bg_consts(th);
    const int warp = threadIdx.x >> 5;
    const long long warps = (long long)gridDim.x * (kBlock / 32);
    for (long long wt = (long long)blockIdx.x * (kBlock / 32) + warp; wt < A.n_items; wt += warps)
    {
        if constexpr (PackedTile<S>::ok)
            warp_tile2<S, FORM, true>(A, th, td, bc, wt, cs[warp], acc);
        else
            warp_tile<S, FORM>(A, th, td, bc, wt, cs[warp], acc);
    }
    reduce_and_store<1 + S>(acc, 1 + th.n_streams, red,
                            partials + (size_t)blockIdx.y * theta_stride + (size_t)blockIdx.x * (1 + th.n_streams));
}

/* The warp-tile integral with tiles handed out by a counter: the warp
 * scheduler favours the older of an SM's two blocks (measured: ~0.42 against
 * ~0.62 ms per tile on the full-size wedge), so a fixed share per warp left
 * one block alone for the last third of the launch.  Each tile's sums are
 * added across the warp in a fixed order and written to the tile's own slot
 * (tile-major, 1 + S components), which the fixed-order reduction then sums:
 * the result does not depend on which warp took which tile. */
template <int S, int FORM>
__global__ void __launch_bounds__(kBlock, MWSEP_F32_MINB) integral_f32w_dyn_kernel(
    const mwsep_area_dev A, const mwsep_theta_consts* __restrict__ thetas, double2* __restrict__ slots,
    long long theta_stride, int* __restrict__ counters, int counter_stride)
{
    __shared__ mwsep_theta_consts th;
    __shared__ ThetaDF<S> td;
    __shared__ __align__(16) float cs[kBlock / 32][TileSmem<S>::N];
    load_theta(th, thetas + blockIdx.y);
    __syncthreads();
    if (mwsep_bg_form(&th) != FORM) return;
    theta_df_part<S>(th, td, (int)threadIdx.x);
    __syncthreads();
    const BgConsts bc = bg_consts(th);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int NC = 1 + th.n_streams;
    int* ctr = counters + (size_t)blockIdx.y * counter_stride;
    double2* out = slots + (size_t)blockIdx.y * theta_stride;
    for (;;)
    {
        int wt = 0;
        if (lane == 0) wt = atomicAdd(ctr, 1);
        wt = __shfl_sync(0xffffffffu, wt, 0);
        if ((long long)wt >= A.n_items) break;
        double acc[1 + S];
#pragma unroll
        for (int k = 0; k < 1 + S; ++k) acc[k] = 0.0;
        if constexpr (PackedTile<S>::ok)
            warp_tile2<S, FORM, true>(A, th, td, bc, wt, cs[warp], acc);
        else
            warp_tile<S, FORM>(A, th, td, bc, wt, cs[warp], acc);
#pragma unroll
        for (int k = 0; k < 1 + S; ++k)
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], off);
        if (lane == 0)
        {
#pragma unroll
            for (int k = 0; k < 1 + S; ++k)
                if (k < NC) out[(size_t)wt * NC + k] = make_double2(acc[k], 0.0);
        }
    }
}

/* calculate_likelihood per star (cpu/evaluation_optimized.c:665-717); the
 * density sums in FP32, everything after them in FP64. */
template <int S>
__global__ void __launch_bounds__(kBlock) likelihood_f32_kernel(const mwsep_stars_dev St,
                                                                const mwsep_theta_consts* __restrict__ thetas,
                                                                const double* __restrict__ integrals,
                                                                double2* __restrict__ partials,
                                                                long long theta_stride)
{
    __shared__ mwsep_theta_consts th;
    __shared__ ThetaDF<S> td;
    __shared__ Log10Sum red[LkSmem<S, kBlock>::N];
    __shared__ LkScale<S> ks;
    load_theta(th, thetas + blockIdx.y);
    __syncthreads();
    const int NS = th.n_streams;
    if (threadIdx.x == 0) lk_scale<S>(th, integrals + (size_t)blockIdx.y * (1 + NS), ks);
    theta_df_part<S>(th, td, (int)threadIdx.x - 32);
    __syncthreads();
    const BgConsts bc = bg_consts(th);

    LkAcc<S> acc;
    acc.init();
    const int N = St.n_stars;
    for (int s0 = blockIdx.x * blockDim.x + threadIdx.x; s0 < N; s0 += gridDim.x * blockDim.x)
        likelihood_star<S>(St, th, td, bc, ks, s0, acc);
    lk_block_store<S>(acc, 3 + NS, red,
                      partials + (size_t)blockIdx.y * theta_stride + (size_t)blockIdx.x * (3 + NS));
}

/* The likelihood in two launches: the per-star densities, which need no
 * integral (so they can run beside the integral kernel), into
 * dens[theta][1 + S][star]; then the epilogue over the integrals, with the
 * fused kernel's grid, star order and reduction (the same bits). */
template <int S>
__global__ void __launch_bounds__(kBlock) likelihood_f32_density_kernel(const mwsep_stars_dev St,
                                                                        const mwsep_theta_consts* __restrict__ thetas,
                                                                        double* __restrict__ dens)
{
    __shared__ mwsep_theta_consts th;
    __shared__ ThetaDF<S> td;
    load_theta(th, thetas + blockIdx.y);
    __syncthreads();
    theta_df_part<S>(th, td, (int)threadIdx.x);
    __syncthreads();
    const BgConsts bc = bg_consts(th);
    const int N = St.n_stars, NS = th.n_streams;
    double* d = dens + (size_t)blockIdx.y * (1 + S) * N;
    for (int s0 = blockIdx.x * blockDim.x + threadIdx.x; s0 < N; s0 += gridDim.x * blockDim.x)
    {
        double bg, st[SArr<S>::N];
        star_density<S>(St, th, td, bc, s0, bg, st);
        d[s0] = bg;
#pragma unroll
        for (int s = 0; s < S; ++s)
            if (s < NS) d[(size_t)(1 + s) * N + s0] = st[s];
    }
}

template <int S>
__global__ void __launch_bounds__(kBlock) likelihood_f32_finish_kernel(int N,
                                                                       const mwsep_theta_consts* __restrict__ thetas,
                                                                       const double* __restrict__ integrals,
                                                                       const double* __restrict__ dens,
                                                                       double2* __restrict__ partials,
                                                                       long long theta_stride)
{
    __shared__ mwsep_theta_consts th;
    __shared__ Log10Sum red[LkSmem<S, kBlock>::N];
    __shared__ LkScale<S> ks;
    load_theta(th, thetas + blockIdx.y);
    __syncthreads();
    const int NS = th.n_streams;
    if (threadIdx.x == 0) lk_scale<S>(th, integrals + (size_t)blockIdx.y * (1 + NS), ks);
    __syncthreads();

    LkAcc<S> acc;
    acc.init();
    const double* d = dens + (size_t)blockIdx.y * (1 + S) * N;
    for (int s0 = blockIdx.x * blockDim.x + threadIdx.x; s0 < N; s0 += gridDim.x * blockDim.x)
    {
        double st[SArr<S>::N];
#pragma unroll
        for (int s = 0; s < S; ++s) st[s] = (s < NS) ? d[(size_t)(1 + s) * N + s0] : 0.0;
        star_epilogue<S>(th, ks, d[s0], st, acc);
    }
    lk_block_store<S>(acc, 3 + NS, red,
                      partials + (size_t)blockIdx.y * theta_stride + (size_t)blockIdx.x * (3 + NS));
}

template <int S>
int launch_integral(const mwsep_area_dev* A, const mwsep_theta_consts* th, const mwsep_launch_shape* sh,
                    int form, double2* partials, cudaStream_t st)
{
    const long long ncomp = 1 + sh->n_streams;
    const long long theta_stride = (long long)sh->n_areas * sh->grid * ncomp;
    double2* base = partials + (size_t)sh->area_index * sh->grid * ncomp;
    dim3 g(sh->grid, sh->n_theta);
    if (A->warp_items)
        switch (form)
        {
        case BG_HERNQUIST: integral_f32w_kernel<S, BG_HERNQUIST><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride); break;
        case BG_HERNQUIST_AUX:
            integral_f32w_kernel<S, BG_HERNQUIST_AUX><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride);
            break;
        case BG_GENERAL: integral_f32w_kernel<S, BG_GENERAL><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride); break;
        default: integral_f32w_kernel<S, BG_NONE><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride); break;
        }
    else
        switch (form)
        {
        case BG_HERNQUIST: integral_f32_kernel<S, BG_HERNQUIST><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride); break;
        case BG_HERNQUIST_AUX:
            integral_f32_kernel<S, BG_HERNQUIST_AUX><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride);
            break;
        case BG_GENERAL: integral_f32_kernel<S, BG_GENERAL><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride); break;
        default: integral_f32_kernel<S, BG_NONE><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride); break;
        }
    return (int)cudaGetLastError();
}

template <int S>
int launch_integral_dyn(const mwsep_area_dev* A, const mwsep_theta_consts* th, const mwsep_launch_shape* sh,
                        long long n_slots, double2* slots, int* counters, cudaStream_t st)
{
    const long long ncomp = 1 + sh->n_streams;
    const long long theta_stride = (long long)sh->n_areas * n_slots * ncomp;
    double2* base = slots + (size_t)sh->area_index * n_slots * ncomp;
    int* ctr = counters + sh->area_index;
    dim3 g(sh->grid, sh->n_theta);
    switch (sh->bg_form)
    {
    case BG_HERNQUIST:
        integral_f32w_dyn_kernel<S, BG_HERNQUIST><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride, ctr, sh->n_areas);
        break;
    case BG_HERNQUIST_AUX:
        integral_f32w_dyn_kernel<S, BG_HERNQUIST_AUX>
            <<<g, kBlock, 0, st>>>(*A, th, base, theta_stride, ctr, sh->n_areas);
        break;
    case BG_GENERAL:
        integral_f32w_dyn_kernel<S, BG_GENERAL><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride, ctr, sh->n_areas);
        break;
    default:
        integral_f32w_dyn_kernel<S, BG_NONE><<<g, kBlock, 0, st>>>(*A, th, base, theta_stride, ctr, sh->n_areas);
        break;
    }
    return (int)cudaGetLastError();
}

template <int S>
int launch_likelihood(const mwsep_stars_dev* St, const mwsep_theta_consts* th, const mwsep_launch_shape* sh,
                      const double* integrals, double2* partials, cudaStream_t st)
{
    const long long theta_stride = (long long)sh->grid * (3 + sh->n_streams);
    dim3 g(sh->grid, sh->n_theta);
    likelihood_f32_kernel<S><<<g, kBlock, 0, st>>>(*St, th, integrals, partials, theta_stride);
    return (int)cudaGetLastError();
}

template <int S>
int launch_density(const mwsep_stars_dev* St, const mwsep_theta_consts* th, const mwsep_launch_shape* sh,
                   double* dens, cudaStream_t st)
{
    dim3 g(sh->grid, sh->n_theta);
    likelihood_f32_density_kernel<S><<<g, kBlock, 0, st>>>(*St, th, dens);
    return (int)cudaGetLastError();
}

template <int S>
int launch_finish(int n_stars, const mwsep_theta_consts* th, const mwsep_launch_shape* sh, const double* integrals,
                  const double* dens, double2* partials, cudaStream_t st)
{
    const long long theta_stride = (long long)sh->grid * (3 + sh->n_streams);
    dim3 g(sh->grid, sh->n_theta);
    likelihood_f32_finish_kernel<S><<<g, kBlock, 0, st>>>(n_stars, th, integrals, dens, partials, theta_stride);
    return (int)cudaGetLastError();
}

/* mwsep_log10_sum_eval's kernel: one block, each thread a strided share */
__global__ void __launch_bounds__(kBlock) log10_sum_kernel(int n, const double* __restrict__ x,
                                                           double2* __restrict__ out)
{
    __shared__ Log10Sum red[LkSmem<0, kBlock>::N];
    LkAcc<0> acc;
    acc.init();
    for (int i = threadIdx.x; i < n; i += blockDim.x) lsum_add(acc.c[0], x[i]);
    lk_block_store<0>(acc, 3, red, out);
}

} // namespace

extern "C" int mwsep_log10_sum_eval(int device, int n, const double* x, double* out)
{
    if (n < 0 || !out || (n > 0 && !x)) return MWSEP_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return MWSEP_ERR_CUDA;
    double* d = nullptr;
    if (cudaMalloc(&d, ((size_t)n + 8) * sizeof(double)) != cudaSuccess)
    {
        cudaGetLastError();
        return MWSEP_ERR_NOMEM;
    }
    double2* o = reinterpret_cast<double2*>(d + n + (n & 1)); /* 16-byte aligned after x */
    cudaError_t e = n > 0 ? cudaMemcpy(d, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice) : cudaSuccess;
    if (e == cudaSuccess)
    {
        log10_sum_kernel<<<1, kBlock>>>(n, d, o);
        e = cudaGetLastError();
    }
    double2 h[1];
    if (e == cudaSuccess) e = cudaMemcpy(h, o, sizeof(double2), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return MWSEP_ERR_CUDA;
    *out = h[0].x;
    return MWSEP_OK;
}

namespace {

template <int S>
cudaError_t f32_occupancy(int* b, int warp_items)
{
    return warp_items ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, integral_f32w_kernel<S, BG_HERNQUIST>, kBlock, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, integral_f32_kernel<S, BG_HERNQUIST>, kBlock, 0);
}

} // namespace

/* Resident blocks per SM of the compensated integral kernel for S streams
 * (sizes the persistent grid); warp_items selects the warp-tile kernel. */
extern "C" int mwsep_integral_f32_blocks_per_sm(int n_streams, int warp_items)
{
    int b = 0;
    cudaError_t e;
    switch (n_streams)
    {
    case 0: e = f32_occupancy<0>(&b, warp_items); break;
    case 1: e = f32_occupancy<1>(&b, warp_items); break;
    case 2: e = f32_occupancy<2>(&b, warp_items); break;
    case 3: e = f32_occupancy<3>(&b, warp_items); break;
    case 4: e = f32_occupancy<4>(&b, warp_items); break;
    default: e = f32_occupancy<8>(&b, warp_items); break;
    }
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return 1;
    }
    return b > 0 ? b : 1;
}

/* shape->block is fixed at kBlock (256) for these kernels. */
extern "C" int mwsep_launch_integral_f32(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                                         const mwsep_launch_shape* sh, double2* partials, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    const int form = sh->bg_form;
    switch (sh->n_streams)
    {
    case 0: return launch_integral<0>(area, th_dev, sh, form, partials, st);
    case 1: return launch_integral<1>(area, th_dev, sh, form, partials, st);
    case 2: return launch_integral<2>(area, th_dev, sh, form, partials, st);
    case 3: return launch_integral<3>(area, th_dev, sh, form, partials, st);
    case 4: return launch_integral<4>(area, th_dev, sh, form, partials, st);
    default: return launch_integral<8>(area, th_dev, sh, form, partials, st);
    }
}

extern "C" int mwsep_launch_integral_f32_dyn(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                                             const mwsep_launch_shape* sh, long long n_slots, double2* slots,
                                             int* counters, void* stream)
{
    if (!area->warp_items) return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    switch (sh->n_streams)
    {
    case 0: return launch_integral_dyn<0>(area, th_dev, sh, n_slots, slots, counters, st);
    case 1: return launch_integral_dyn<1>(area, th_dev, sh, n_slots, slots, counters, st);
    case 2: return launch_integral_dyn<2>(area, th_dev, sh, n_slots, slots, counters, st);
    case 3: return launch_integral_dyn<3>(area, th_dev, sh, n_slots, slots, counters, st);
    case 4: return launch_integral_dyn<4>(area, th_dev, sh, n_slots, slots, counters, st);
    default: return launch_integral_dyn<8>(area, th_dev, sh, n_slots, slots, counters, st);
    }
}

extern "C" int mwsep_launch_likelihood_f32(const mwsep_stars_dev* stars, const mwsep_theta_consts* th_dev,
                                           const mwsep_launch_shape* sh, const double* integrals,
                                           double2* partials, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    switch (sh->n_streams)
    {
    case 0: return launch_likelihood<0>(stars, th_dev, sh, integrals, partials, st);
    case 1: return launch_likelihood<1>(stars, th_dev, sh, integrals, partials, st);
    case 2: return launch_likelihood<2>(stars, th_dev, sh, integrals, partials, st);
    case 3: return launch_likelihood<3>(stars, th_dev, sh, integrals, partials, st);
    case 4: return launch_likelihood<4>(stars, th_dev, sh, integrals, partials, st);
    default: return launch_likelihood<8>(stars, th_dev, sh, integrals, partials, st);
    }
}

extern "C" int mwsep_launch_likelihood_f32_density(const mwsep_stars_dev* stars, const mwsep_theta_consts* th_dev,
                                                   const mwsep_launch_shape* sh, double* dens, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    switch (sh->n_streams)
    {
    case 0: return launch_density<0>(stars, th_dev, sh, dens, st);
    case 1: return launch_density<1>(stars, th_dev, sh, dens, st);
    case 2: return launch_density<2>(stars, th_dev, sh, dens, st);
    case 3: return launch_density<3>(stars, th_dev, sh, dens, st);
    case 4: return launch_density<4>(stars, th_dev, sh, dens, st);
    default: return launch_density<8>(stars, th_dev, sh, dens, st);
    }
}

extern "C" int mwsep_launch_likelihood_f32_finish(int n_stars, const mwsep_theta_consts* th_dev,
                                                  const mwsep_launch_shape* sh, const double* integrals,
                                                  const double* dens, double2* partials, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    switch (sh->n_streams)
    {
    case 0: return launch_finish<0>(n_stars, th_dev, sh, integrals, dens, partials, st);
    case 1: return launch_finish<1>(n_stars, th_dev, sh, integrals, dens, partials, st);
    case 2: return launch_finish<2>(n_stars, th_dev, sh, integrals, dens, partials, st);
    case 3: return launch_finish<3>(n_stars, th_dev, sh, integrals, dens, partials, st);
    case 4: return launch_finish<4>(n_stars, th_dev, sh, integrals, dens, partials, st);
    default: return launch_finish<8>(n_stars, th_dev, sh, integrals, dens, partials, st);
    }
}

MWSEP_CHECKS_READER(mwsep_checks_f32)
