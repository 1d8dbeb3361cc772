/* mwsep_engine_f32.cu -- compensated-FP32 kernels of the tiled engine.
 *
 * One persistent launch evaluates every request of a batch, whatever wedge
 * each names: warps (integrals) and blocks (likelihood) take (request, area,
 * item-run) tiles from a global counter, so uneven wedges balance
 * themselves, and each tile writes its own partial slot, so a request's
 * result does not depend on which warp ran which tile or what else was in
 * the batch.  Per tile the block dispatches on
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

/* 8-byte words from src to dst by the 32 lanes of a warp */
__device__ __forceinline__ void warp_copy(void* dst, const void* src, int bytes)
{
    static_assert(sizeof(mwsep_area_dev) % 8 == 0 && sizeof(mwsep_theta_consts) % 8 == 0,
                  "descriptors are copied in 8-byte words");
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(dst);
    for (int i = threadIdx.x & 31; i < bytes / 8; i += 32) d[i] = s[i];
}

/* A warp's shared memory in the integral kernel: the column constants of its
 * current warp tile, and its integral tile's theta, area and theta pairs. */
template <int S>
struct WarpSlot
{
    __align__(16) float cs[TileSmem<S>::N];
    mwsep_theta_consts th;
    mwsep_area_dev A;
    ThetaDF<S> td;
};

/* One integral tile by one warp: its warp tiles in order (or its thread
 * items, the lanes striding), then the lanes' sums added across the warp in
 * a fixed order into the tile's slot. */
template <int S, int FORM>
__device__ __forceinline__ void itile(const mwsep_area_dev& A, const mwsep_theta_consts& th, const ThetaDF<S>& td,
                                      const mwsep_itile& t, float* cs, double2* out)
{
    double acc[1 + S];
#pragma unroll
    for (int k = 0; k < 1 + S; ++k) acc[k] = 0.0;
    const BgConsts bc = bg_consts(th);
    if (A.warp_items)
    {
        for (long long wt = t.item_begin; wt < t.item_end; ++wt)
        {
            if constexpr (PackedTile<S>::ok)
                warp_tile2<S, FORM>(A, th, td, bc, wt, cs, acc);
            else
                warp_tile<S, FORM>(A, th, td, bc, wt, cs, acc);
        }
    }
    else
        for (long long item = t.item_begin + (threadIdx.x & 31); item < t.item_end; item += 32)
            integral_item<S, FORM>(A, th, bc, item, acc);
#pragma unroll
    for (int k = 0; k < 1 + S; ++k)
        for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], off);
    if ((threadIdx.x & 31) == 0)
    {
#pragma unroll
        for (int k = 0; k < 1 + S; ++k)
            if (k < 1 + th.n_streams) out[k] = make_double2(acc[k], 0.0);
    }
}

template <int S>
__device__ __forceinline__ void itile_form(const mwsep_area_dev& A, const mwsep_theta_consts& th,
                                           const ThetaDF<S>& td, const mwsep_itile& t, float* cs, double2* out)
{
    switch (mwsep_bg_form(&th))
    {
    case BG_HERNQUIST: itile<S, BG_HERNQUIST>(A, th, td, t, cs, out); break;
    case BG_HERNQUIST_AUX: itile<S, BG_HERNQUIST_AUX>(A, th, td, t, cs, out); break;
    case BG_GENERAL: itile<S, BG_GENERAL>(A, th, td, t, cs, out); break;
    default: itile<S, BG_NONE>(A, th, td, t, cs, out); break;
    }
}

/* Streams handled by a kernel of group G: exactly G up to 4, 8 (with
 * guards) for group 5. */
template <int G>
struct GroupS
{
    static constexpr int S = G <= 4 ? G : 8;
};

template <int G>
constexpr size_t integral_smem()
{
    return sizeof(WarpSlot<GroupS<G>::S>) * (kBlock / 32);
}

/* Each warp takes integral tiles from the group's counter on its own (a
 * block-wide tile waited at its end for its slowest warp: a half-width
 * warp tile at a wedge's mu edge left the other seven warps of the block
 * idle for half a tile), with its tile's theta and area in its own slot of
 * shared memory. */
template <int G>
__global__ void __launch_bounds__(kBlock, 2) engine_integral_f32_kernel(const mwsep_engine_args a)
{
    constexpr int S = GroupS<G>::S;
    extern __shared__ __align__(16) unsigned char smem[];
    WarpSlot<S>& ws = reinterpret_cast<WarpSlot<S>*>(smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int n_tiles = a.counters[4 * G + 2];
    for (;;)
    {
        int t = 0;
        if (lane == 0) t = atomicAdd(&a.counters[4 * G + 0], 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n_tiles) break;
        const mwsep_itile tile = a.itiles[t];
        warp_copy(&ws.th, a.thetas + MWSEP_IDX(tile.req, a.counters[MWSEP_ENG_NREQ], 10), sizeof(mwsep_theta_consts));
        warp_copy(&ws.A, a.areas + MWSEP_IDX(tile.area_desc, a.n_area_desc, 11), sizeof(mwsep_area_dev));
        __syncwarp();
        theta_df_part<S>(ws.th, ws.td, lane);
        __syncwarp();
        itile_form<S>(ws.A, ws.th, ws.td, tile, ws.cs, a.ipart + (size_t)t * MWSEP_ENG_ICOMP);
        __syncwarp();
    }
}

template <int S>
__device__ __forceinline__ void ltile(const mwsep_stars_dev& St, const mwsep_theta_consts& th,
                                      const ThetaDF<S>& td, const LkScale<S>& ks, const mwsep_ltile& t,
                                      Log10Sum* red, double2* out)
{
    LkAcc<S> acc;
    acc.init();
    const BgConsts bc = bg_consts(th);
    for (int s0 = t.star_begin + threadIdx.x; s0 < t.star_end; s0 += blockDim.x)
        likelihood_star<S>(St, th, td, bc, ks, s0, acc);
    lk_block_store<S>(acc, 3 + th.n_streams, red, out);
}

template <int G>
__global__ void __launch_bounds__(kBlock, 2) engine_likelihood_f32_kernel(const mwsep_engine_args a)
{
    constexpr int S = GroupS<G>::S;
    __shared__ mwsep_theta_consts th;
    __shared__ ThetaDF<S> td;
    __shared__ Log10Sum red[LkSmem<S, kBlock>::N];
    __shared__ LkScale<S> ks;
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
        if (threadIdx.x == 0) lk_scale<S>(th, I, ks);
        theta_df_part<S>(th, td, (int)threadIdx.x - 32);
        __syncthreads();
        double2* out = a.lpart + (size_t)t * MWSEP_ENG_LCOMP;
        ltile<S>(St, th, td, ks, tile, red, out);
        __syncthreads();
    }
}

} // namespace

namespace {

/* the integral kernel's per-warp slots can pass the 48 KB of a default
 * launch (four streams: ~53 KB per block) */
template <int G>
cudaError_t integral_smem_attr()
{
    static_assert(integral_smem<G>() <= 100 * 1024, "two blocks per SM must fit in shared memory");
    return cudaFuncSetAttribute(engine_integral_f32_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)integral_smem<G>());
}

template <int G>
void launch_group(int phase, const mwsep_engine_args* a, int grid, cudaStream_t st)
{
    if (phase == 0)
    {
        if (integral_smem_attr<G>() != cudaSuccess) return;
        engine_integral_f32_kernel<G><<<grid, kBlock, integral_smem<G>(), st>>>(*a);
    }
    else
        engine_likelihood_f32_kernel<G><<<grid, kBlock, 0, st>>>(*a);
}

template <int G>
cudaError_t group_occupancy(int* b, int phase)
{
    if (phase != 0)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, engine_likelihood_f32_kernel<G>, kBlock, 0);
    const cudaError_t e = integral_smem_attr<G>();
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, engine_integral_f32_kernel<G>, kBlock, integral_smem<G>());
}

} // namespace

extern "C" int mwsep_engine_f32_launch(int phase, int group, const mwsep_engine_args* a, int grid, void* stream)
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

extern "C" int mwsep_engine_f32_blocks_per_sm(int phase, int group)
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

MWSEP_CHECKS_READER(mwsep_checks_engine_f32)
