/* mwsep_engine_f32.cu -- compensated-FP32 kernels of the tiled engine.
 *
 * One persistent launch evaluates every request of a batch, whatever wedge
 * each names: blocks take (request, area, item-run) tiles from a global
 * counter, so uneven wedges balance themselves, and each tile writes its own
 * partial slot, so a request's result does not depend on which block ran
 * which tile or what else was in the batch.  Per tile the block dispatches on
 * the request's stream count and background form to the same specialised
 * density code as the single-wedge kernels (mwsep_f32_point.cuh).
 */
#include <cuda_runtime.h>
#include "mwsep_internal.h"
#include "mwsep_reduce.cuh"
#include "mwsep_f32_point.cuh"

namespace {

using namespace mwsep::f32;

constexpr int kBlock = 256;

__device__ __forceinline__ void load_area(mwsep_area_dev& dst, const mwsep_area_dev* src)
{
    static_assert(sizeof(mwsep_area_dev) % 8 == 0, "area descriptor must be 8-byte sized");
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(mwsep_area_dev) / 8); i += blockDim.x) d[i] = s[i];
}

/* cs: the block's column-constant scratch, kTileCols * ColWords<S>::N floats
 * per warp (used by warp-tile items). */
template <int S, int FORM>
__device__ __forceinline__ void itile(const mwsep_area_dev& A, const mwsep_theta_consts& th, const mwsep_itile& t,
                                      double* red, float* cs, double2* out)
{
    double acc[1 + S];
#pragma unroll
    for (int k = 0; k < 1 + S; ++k) acc[k] = 0.0;
    const BgConsts bc = bg_consts(th);
    if (A.warp_items)
    {
        const int warp = threadIdx.x >> 5;
        constexpr int CW = PackedTile<S>::ok ? PackedTile<S>::W : ColWords<S>::N;
        float* mine = cs + warp * mwsep::kTileCols * CW;
        for (long long wt = t.item_begin + warp; wt < t.item_end; wt += blockDim.x >> 5)
        {
            if constexpr (PackedTile<S>::ok)
                warp_tile2<S, FORM>(A, th, bc, wt, mine, acc);
            else
                warp_tile<S, FORM>(A, th, bc, wt, mine, acc);
        }
    }
    else
        for (long long item = t.item_begin + threadIdx.x; item < t.item_end; item += blockDim.x)
            integral_item<S, FORM>(A, th, bc, item, acc);
    reduce_and_store<1 + S>(acc, 1 + th.n_streams, red, out);
}

template <int S>
__device__ __forceinline__ void itile_form(const mwsep_area_dev& A, const mwsep_theta_consts& th,
                                           const mwsep_itile& t, double* red, float* cs, double2* out)
{
    switch (mwsep_bg_form(&th))
    {
    case BG_HERNQUIST: itile<S, BG_HERNQUIST>(A, th, t, red, cs, out); break;
    case BG_HERNQUIST_AUX: itile<S, BG_HERNQUIST_AUX>(A, th, t, red, cs, out); break;
    case BG_GENERAL: itile<S, BG_GENERAL>(A, th, t, red, cs, out); break;
    default: itile<S, BG_NONE>(A, th, t, red, cs, out); break;
    }
}

template <int CLS>
__global__ void __launch_bounds__(kBlock, 2) engine_integral_f32_kernel(const mwsep_engine_args a)
{
    __shared__ mwsep_theta_consts th;
    __shared__ mwsep_area_dev A;
    __shared__ double red[2 * (CLS == 0 ? 5 : MWSEP_ENG_ICOMP) * 32];
    __shared__ __align__(16) float cs[(kBlock / 32) * mwsep::kTileCols *
                                      (CLS == 0 ? PackedTile<4>::W : ColWords<8>::N)];
    __shared__ int s_tile;
    const int n_tiles = a.counters[4 * CLS + 2];
    for (;;)
    {
        if (threadIdx.x == 0) s_tile = atomicAdd(&a.counters[4 * CLS + 0], 1);
        __syncthreads();
        const int t = s_tile;
        if (t >= n_tiles) break;
        const mwsep_itile tile = a.itiles[t];
        load_theta(th, a.thetas + MWSEP_IDX(tile.req, a.counters[MWSEP_ENG_NREQ], 10));
        load_area(A, a.areas + MWSEP_IDX(tile.area_desc, a.n_area_desc, 11));
        __syncthreads();
        double2* out = a.ipart + (size_t)t * MWSEP_ENG_ICOMP;
        if (CLS == 1)
            itile_form<8>(A, th, tile, red, cs, out);
        else
            switch (th.n_streams)
            {
            case 0: itile_form<0>(A, th, tile, red, cs, out); break;
            case 1: itile_form<1>(A, th, tile, red, cs, out); break;
            case 2: itile_form<2>(A, th, tile, red, cs, out); break;
            case 3: itile_form<3>(A, th, tile, red, cs, out); break;
            default: itile_form<4>(A, th, tile, red, cs, out); break;
            }
        __syncthreads();
    }
}

template <int S>
__device__ __forceinline__ void ltile(const mwsep_stars_dev& St, const mwsep_theta_consts& th, const double* I,
                                      const mwsep_ltile& t, double* red, double2* out)
{
    double acc[3 + S];
#pragma unroll
    for (int k = 0; k < 3 + S; ++k) acc[k] = 0.0;
    const BgConsts bc = bg_consts(th);
    for (int s0 = t.star_begin + threadIdx.x; s0 < t.star_end; s0 += blockDim.x)
        likelihood_star<S>(St, th, bc, I, s0, acc);
    reduce_and_store<3 + S>(acc, 3 + th.n_streams, red, out);
}

template <int CLS>
__global__ void __launch_bounds__(kBlock, 2) engine_likelihood_f32_kernel(const mwsep_engine_args a)
{
    __shared__ mwsep_theta_consts th;
    __shared__ double red[2 * (CLS == 0 ? 7 : MWSEP_ENG_LCOMP) * 32];
    __shared__ int s_tile;
    const int n_tiles = a.counters[4 * CLS + 3];
    for (;;)
    {
        if (threadIdx.x == 0) s_tile = atomicAdd(&a.counters[4 * CLS + 1], 1);
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
        if (CLS == 1)
            ltile<8>(St, th, I, tile, red, out);
        else
            switch (th.n_streams)
            {
            case 0: ltile<0>(St, th, I, tile, red, out); break;
            case 1: ltile<1>(St, th, I, tile, red, out); break;
            case 2: ltile<2>(St, th, I, tile, red, out); break;
            case 3: ltile<3>(St, th, I, tile, red, out); break;
            default: ltile<4>(St, th, I, tile, red, out); break;
            }
        __syncthreads();
    }
}

} // namespace

extern "C" int mwsep_engine_f32_launch(int phase, int cls, const mwsep_engine_args* a, int grid, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (phase == 0 && cls == 0) engine_integral_f32_kernel<0><<<grid, kBlock, 0, st>>>(*a);
    else if (phase == 0) engine_integral_f32_kernel<1><<<grid, kBlock, 0, st>>>(*a);
    else if (cls == 0) engine_likelihood_f32_kernel<0><<<grid, kBlock, 0, st>>>(*a);
    else engine_likelihood_f32_kernel<1><<<grid, kBlock, 0, st>>>(*a);
    return (int)cudaGetLastError();
}

extern "C" int mwsep_engine_f32_blocks_per_sm(int phase, int cls)
{
    int b = 0;
    cudaError_t e;
    if (phase == 0 && cls == 0) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, engine_integral_f32_kernel<0>, kBlock, 0);
    else if (phase == 0) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, engine_integral_f32_kernel<1>, kBlock, 0);
    else if (cls == 0) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, engine_likelihood_f32_kernel<0>, kBlock, 0);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, engine_likelihood_f32_kernel<1>, kBlock, 0);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return 1;
    }
    return b > 0 ? b : 1;
}

MWSEP_CHECKS_READER(mwsep_checks_engine_f32)
