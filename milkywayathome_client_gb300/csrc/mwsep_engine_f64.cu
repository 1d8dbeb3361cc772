/* mwsep_engine_f64.cu -- plain-FP64 kernels of the tiled engine (same tile
 * scheme as mwsep_engine_f32.cu; density arithmetic of mwsep_f64_point.cuh,
 * compiled with -fmad=false). */
#include <cuda_runtime.h>
#include "mwsep_internal.h"
#include "mwsep_reduce.cuh"
#include "mwsep_f64_point.cuh"

namespace {

using namespace mwsep::f64;
using mwsep::comp_sum;

constexpr int kBlock = 256;

__device__ __forceinline__ void load_area(mwsep_area_dev& dst, const mwsep_area_dev* src)
{
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(mwsep_area_dev) / 8); i += blockDim.x) d[i] = s[i];
}

template <int NC>
__device__ __forceinline__ void store_partial(comp_sum (&acc)[NC], int ncomp, double* red, double2* out)
{
    mwsep::block_reduce<NC>(acc, red);
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int k = 0; k < NC; ++k)
            if (k < ncomp) out[k] = make_double2(acc[k].s, acc[k].c);
    }
}

template <int SMAX>
__device__ __forceinline__ void itile(const mwsep_area_dev& A, const mwsep_theta_consts& th, const double* etab,
                                      const mwsep_itile& t, double* red, double2* out)
{
    comp_sum acc[1 + SMAX];
#pragma unroll
    for (int k = 0; k < 1 + SMAX; ++k) acc[k].zero();
    for (long long item = t.item_begin + threadIdx.x; item < t.item_end; item += blockDim.x)
        integral_item<SMAX>(A, th, etab, item, acc);
    store_partial<1 + SMAX>(acc, 1 + th.n_streams, red, out);
}

/* The FP64 kernels are specialised on a bound of the stream count: group G
 * (the stream count up to 4, or 5 for 5..8) runs with SMAX = 1, 1, 2, 4, 4, 8. */
template <int G>
struct GroupSmax
{
    static constexpr int S = G <= 1 ? 1 : G == 2 ? 2 : G <= 4 ? 4 : 8;
};

template <int G>
__global__ void __launch_bounds__(kBlock) engine_integral_f64_kernel(const mwsep_engine_args a)
{
    constexpr int SMAX = GroupSmax<G>::S;
    __shared__ mwsep_theta_consts th;
    __shared__ mwsep_area_dev A;
    __shared__ double red[2 * (1 + SMAX) * 32];
    __shared__ double etab[kExpTable];
    __shared__ int s_tile;
    const int n_tiles = a.counters[4 * G + 2];
    exp_tang_table(etab);
    for (;;)
    {
        if (threadIdx.x == 0) s_tile = atomicAdd(&a.counters[4 * G + 0], 1);
        __syncthreads();
        const int t = s_tile;
        if (t >= n_tiles) break;
        const mwsep_itile tile = a.itiles[t];
        load_theta(th, a.thetas + MWSEP_IDX(tile.req, a.counters[MWSEP_ENG_NREQ], 10));
        load_area(A, a.areas + MWSEP_IDX(tile.area_desc, a.n_area_desc, 11));
        __syncthreads();
        double2* out = a.ipart + (size_t)t * MWSEP_ENG_ICOMP;
        itile<SMAX>(A, th, etab, tile, red, out);
        __syncthreads();
    }
}

template <int SMAX>
__device__ __forceinline__ void ltile(const mwsep_stars_dev& St, const mwsep_theta_consts& th, const double* I,
                                      const mwsep_ltile& t, double* red, double2* out)
{
    comp_sum acc[3 + SMAX];
#pragma unroll
    for (int k = 0; k < 3 + SMAX; ++k) acc[k].zero();
    for (int s0 = t.star_begin + threadIdx.x; s0 < t.star_end; s0 += blockDim.x)
        likelihood_star<SMAX>(St, th, I, s0, acc);
    store_partial<3 + SMAX>(acc, 3 + th.n_streams, red, out);
}

template <int G>
__global__ void __launch_bounds__(kBlock) engine_likelihood_f64_kernel(const mwsep_engine_args a)
{
    constexpr int SMAX = GroupSmax<G>::S;
    __shared__ mwsep_theta_consts th;
    __shared__ double red[2 * (3 + SMAX) * 32];
    __shared__ int s_tile;
    const int n_tiles = a.counters[4 * G + 3];
    for (;;)
    {
        if (threadIdx.x == 0) s_tile = atomicAdd(&a.counters[4 * G + 1], 1);
        __syncthreads();
        const int t = s_tile;
        if (t >= n_tiles) break;
        const mwsep_ltile tile = a.ltiles[t];
        load_theta(th, a.thetas + MWSEP_IDX(tile.req, a.counters[MWSEP_ENG_NREQ], 10));
        __syncthreads();
        const mwsep_stars_dev St =
            a.stars[MWSEP_IDX(a.reqs[MWSEP_IDX(tile.req, a.counters[MWSEP_ENG_NREQ], 10)].stars, a.n_star_desc, 12)];
        const double* I = a.out + (size_t)tile.req * MWSEP_ENG_OUT_STRIDE + MWSEP_ENG_OUT_INTS;
        double2* out = a.lpart + (size_t)t * MWSEP_ENG_LCOMP;
        ltile<SMAX>(St, th, I, tile, red, out);
        __syncthreads();
    }
}

} // namespace

namespace {

template <int G>
void launch_group(int phase, const mwsep_engine_args* a, int grid, cudaStream_t st)
{
    if (phase == 0)
        engine_integral_f64_kernel<G><<<grid, kBlock, 0, st>>>(*a);
    else
        engine_likelihood_f64_kernel<G><<<grid, kBlock, 0, st>>>(*a);
}

template <int G>
cudaError_t group_occupancy(int* b, int phase)
{
    return phase == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, engine_integral_f64_kernel<G>, kBlock, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, engine_likelihood_f64_kernel<G>, kBlock, 0);
}

} // namespace

extern "C" int mwsep_engine_f64_launch(int phase, int group, const mwsep_engine_args* a, int grid, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    switch (group)
    {
    case 0: launch_group<0>(phase, a, grid, st); break;
    case 1: launch_group<1>(phase, a, grid, st); break;
    case 2: launch_group<2>(phase, a, grid, st); break;
    case 3: launch_group<3>(phase, a, grid, st); break;
    case 4: launch_group<4>(phase, a, grid, st); break;
    default: launch_group<5>(phase, a, grid, st); break;
    }
    return (int)cudaGetLastError();
}

extern "C" int mwsep_engine_f64_blocks_per_sm(int phase, int group)
{
    int b = 0;
    cudaError_t e;
    switch (group)
    {
    case 0: e = group_occupancy<0>(&b, phase); break;
    case 1: e = group_occupancy<1>(&b, phase); break;
    case 2: e = group_occupancy<2>(&b, phase); break;
    case 3: e = group_occupancy<3>(&b, phase); break;
    case 4: e = group_occupancy<4>(&b, phase); break;
    default: e = group_occupancy<5>(&b, phase); break;
    }
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return 1;
    }
    return b > 0 ? b : 1;
}

MWSEP_CHECKS_READER(mwsep_checks_engine_f64)
