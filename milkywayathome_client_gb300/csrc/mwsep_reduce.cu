/* mwsep_reduce.cu -- fixed-order reductions of the per-block compensated
 * partials.  One block per (component, theta), so the components reduce
 * side by side; each thread walks a fixed stride of the partials, then the
 * block combines error-free.  The result of a theta depends only on its own
 * partials and the grid size, never on what else shares the launch. */
#include <cuda_runtime.h>
#include "mwsep_internal.h"
#include "mwsep_reduce.cuh"

using mwsep::comp_sum;

namespace {

constexpr int kReduceThreads = 256;

/* Area integrals = sum over blocks (pair value s + c), then
 * I = I_0 - sum_{a>=1} I_a in area order (cpu/evaluation_optimized.c:584-593). */
__global__ void __launch_bounds__(kReduceThreads)
    reduce_integrals_kernel(const double2* __restrict__ partials, int n_areas, int grid, int ncomp,
                            double* __restrict__ out_areas, double* __restrict__ out_integrals)
{
    /* block (c, t): component c of parameter vector t, every area, then
     * I_c = I_c(area 0) - sum of the cut areas' (each component's order is
     * independent of the others') */
    __shared__ double red[2 * 32];
    const int c = blockIdx.x, t = blockIdx.y;
    const double2* base = partials + (size_t)t * n_areas * grid * ncomp;
    double* areas = out_areas + (size_t)t * n_areas * ncomp;
    for (int a = 0; a < n_areas; ++a)
    {
        comp_sum acc[1];
        acc[0].zero();
        for (int b = threadIdx.x; b < grid; b += blockDim.x)
        {
            const double2 v = base[((size_t)a * grid + b) * ncomp + c];
            acc[0].merge(v.x, v.y);
        }
        mwsep::block_reduce<1>(acc, red);
        if (threadIdx.x == 0) areas[a * ncomp + c] = acc[0].s + acc[0].c;
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        double I = areas[c];
        for (int a = 1; a < n_areas; ++a) I -= areas[a * ncomp + c];
        out_integrals[(size_t)t * ncomp + c] = I;
    }
}

__global__ void __launch_bounds__(kReduceThreads)
    reduce_likelihood_kernel(const double2* __restrict__ partials, int grid, int nslots, double* __restrict__ out)
{
    /* block (c, t): slot c of parameter vector t */
    __shared__ double red[2 * 32];
    const int c = blockIdx.x, t = blockIdx.y;
    const double2* base = partials + (size_t)t * grid * nslots;
    comp_sum acc[1];
    acc[0].zero();
    for (int b = threadIdx.x; b < grid; b += blockDim.x)
    {
        const double2 v = base[(size_t)b * nslots + c];
        acc[0].merge(v.x, v.y);
    }
    mwsep::block_reduce<1>(acc, red);
    if (threadIdx.x == 0) out[(size_t)t * nslots + c] = acc[0].s + acc[0].c;
}

/* First level for per-tile slots: block (c + ncomp * g, row) sums component
 * c of slots [g * seg_len, (g + 1) * seg_len) of row (theta * n_areas + area)
 * into seg[(row * n_seg + g) * ncomp + c], a fixed segmentation. */
__global__ void __launch_bounds__(kReduceThreads)
    reduce_slots_kernel(const double2* __restrict__ slots, long long n_slots, int seg_len, int n_seg, int ncomp,
                        double2* __restrict__ seg)
{
    __shared__ double red[2 * 32];
    const int c = blockIdx.x % ncomp, g = blockIdx.x / ncomp;
    const size_t row = blockIdx.y;
    const double2* base = slots + row * (size_t)n_slots * ncomp;
    const long long b0 = (long long)g * seg_len;
    const long long b1 = b0 + seg_len < n_slots ? b0 + seg_len : n_slots;
    comp_sum acc[1];
    acc[0].zero();
    for (long long b = b0 + threadIdx.x; b < b1; b += blockDim.x)
    {
        const double2 v = base[(size_t)b * ncomp + c];
        acc[0].merge(v.x, v.y);
    }
    mwsep::block_reduce<1>(acc, red);
    if (threadIdx.x == 0) seg[(row * n_seg + g) * ncomp + c] = make_double2(acc[0].s, acc[0].c);
}

} // namespace

extern "C" int mwsep_launch_reduce_slots(const double2* slots, int n_rows, long long n_slots, int ncomp, int seg_len,
                                         double2* seg, void* stream)
{
    const int n_seg = (int)((n_slots + seg_len - 1) / seg_len);
    if (n_rows < 1 || n_rows > 65535 || n_seg < 1 || (long long)n_seg * ncomp > 2147483647LL)
        return (int)cudaErrorInvalidValue;
    reduce_slots_kernel<<<dim3(n_seg * ncomp, n_rows), kReduceThreads, 0, (cudaStream_t)stream>>>(
        slots, n_slots, seg_len, n_seg, ncomp, seg);
    return (int)cudaGetLastError();
}

extern "C" int mwsep_launch_reduce_integrals(const double2* partials, const mwsep_launch_shape* sh,
                                             double* out_areas, double* out_integrals, void* stream)
{
    reduce_integrals_kernel<<<dim3(1 + sh->n_streams, sh->n_theta), kReduceThreads, 0, (cudaStream_t)stream>>>(
        partials, sh->n_areas, sh->grid, 1 + sh->n_streams, out_areas, out_integrals);
    return (int)cudaGetLastError();
}

extern "C" int mwsep_launch_reduce_likelihood(const double2* partials, const mwsep_launch_shape* sh, double* out,
                                              void* stream)
{
    reduce_likelihood_kernel<<<dim3(3 + sh->n_streams, sh->n_theta), kReduceThreads, 0, (cudaStream_t)stream>>>(
        partials, sh->grid, 3 + sh->n_streams, out);
    return (int)cudaGetLastError();
}

/* ---- tiled engine: per-request fixed-order reductions ---- */

namespace {

/* Sum the tile partials [t0, t1) (stride `stride`, component c) of one
 * request in a fixed order: thread-strided, then the block tree. */
__device__ double sum_tiles(const double2* part, int stride, int c, int t0, int t1, double* red)
{
    comp_sum acc[1];
    acc[0].zero();
    for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x)
    {
        const double2 v = part[(size_t)t * stride + c];
        acc[0].merge(v.x, v.y);
    }
    mwsep::block_reduce<1>(acc, red);
    double r = acc[0].s + acc[0].c;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kReduceThreads) engine_reduce_integrals_kernel(const mwsep_engine_args a)
{
    __shared__ double red[2 * 32];
    const int n_req = a.counters[MWSEP_ENG_NREQ];
    for (int r = blockIdx.x; r < n_req; r += gridDim.x)
    {
        const mwsep_req_dev q = a.reqs[r];
        const int ncomp = 1 + q.n_streams;
        double* out = a.out + (size_t)r * MWSEP_ENG_OUT_STRIDE;
        for (int ar = 0; ar < q.n_areas; ++ar)
            for (int c = 0; c < ncomp; ++c)
            {
                const double v = sum_tiles(a.ipart, MWSEP_ENG_ICOMP, c, q.area_slot[ar], q.area_slot[ar + 1], red);
                if (threadIdx.x == 0) out[MWSEP_ENG_OUT_AREAS + ar * MWSEP_ENG_ICOMP + c] = v;
            }
        __syncthreads();
        if (threadIdx.x == 0)
        {
            /* cpu/evaluation_optimized.c:584-593 */
            for (int c = 0; c < ncomp; ++c)
            {
                double I = out[MWSEP_ENG_OUT_AREAS + c];
                for (int ar = 1; ar < q.n_areas; ++ar) I -= out[MWSEP_ENG_OUT_AREAS + ar * MWSEP_ENG_ICOMP + c];
                out[MWSEP_ENG_OUT_INTS + c] = I;
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kReduceThreads) engine_reduce_likelihood_kernel(const mwsep_engine_args a)
{
    __shared__ double red[2 * 32];
    const int n_req = a.counters[MWSEP_ENG_NREQ];
    for (int r = blockIdx.x; r < n_req; r += gridDim.x)
    {
        const mwsep_req_dev q = a.reqs[r];
        double* out = a.out + (size_t)r * MWSEP_ENG_OUT_STRIDE + MWSEP_ENG_OUT_LK;
        for (int c = 0; c < 3 + q.n_streams; ++c)
        {
            const double v = sum_tiles(a.lpart, MWSEP_ENG_LCOMP, c, q.lk_slot0, q.lk_slot1, red);
            if (threadIdx.x == 0) out[c] = v;
        }
    }
}

} // namespace

extern "C" int mwsep_engine_reduce(int phase, const mwsep_engine_args* a, int grid, void* stream)
{
    if (phase == 0)
        engine_reduce_integrals_kernel<<<grid, kReduceThreads, 0, (cudaStream_t)stream>>>(*a);
    else
        engine_reduce_likelihood_kernel<<<grid, kReduceThreads, 0, (cudaStream_t)stream>>>(*a);
    return (int)cudaGetLastError();
}
