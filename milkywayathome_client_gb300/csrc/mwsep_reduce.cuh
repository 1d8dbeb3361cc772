/* mwsep_reduce.cuh -- compensated (double-double style) sums used by every
 * kernel: per-thread Kahan accumulation as in the reference
 * (cpu/evaluation_optimized.c:506-519, 682-684, 708-710), then error-free
 * pairwise combination across lanes, warps and blocks, so the order of
 * every reduction is fixed by the launch shape alone (no atomics). */
#ifndef MWSEP_REDUCE_CUH
#define MWSEP_REDUCE_CUH

#include <cuda_runtime.h>

namespace mwsep {

/* Knuth's TwoSum: s + e == a + b exactly.  The arithmetic is spelled with
 * the _rn intrinsics so no contraction can merge its steps. */
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e)
{
    s = __dadd_rn(a, b);
    const double bb = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

/* A compensated accumulator; value = s + c. */
struct comp_sum
{
    double s, c;
    __device__ __forceinline__ void zero() { s = 0.0; c = 0.0; }
    /* Kahan step in the reference's form. */
    __device__ __forceinline__ void add(double x)
    {
        const double t = s;
        s = __dadd_rn(s, x);
        c = __dadd_rn(c, __dsub_rn(x, __dsub_rn(s, t)));
    }
    /* Merge another accumulator, error-free in the leading part. */
    __device__ __forceinline__ void merge(double os, double oc)
    {
        double hi, e;
        two_sum(s, os, hi, e);
        double lo = __dadd_rn(__dadd_rn(c, oc), e);
        two_sum(hi, lo, s, c);
    }
};

/* Reduce NC compensated accumulators across a block of blockDim.x threads
 * (a multiple of 32, at most 1024).  Block result is valid in thread 0.
 * smem must hold 2*NC*32 doubles. */
template <int NC>
__device__ __forceinline__ void block_reduce(comp_sum (&acc)[NC], double* smem)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NC; ++k)
    {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
        {
            const double os = __shfl_down_sync(0xffffffffu, acc[k].s, off);
            const double oc = __shfl_down_sync(0xffffffffu, acc[k].c, off);
            if (lane < off) acc[k].merge(os, oc);
        }
    }
    if (lane == 0)
    {
#pragma unroll
        for (int k = 0; k < NC; ++k)
        {
            smem[(k * 32 + warp) * 2 + 0] = acc[k].s;
            smem[(k * 32 + warp) * 2 + 1] = acc[k].c;
        }
    }
    __syncthreads();
    if (warp == 0)
    {
#pragma unroll
        for (int k = 0; k < NC; ++k)
        {
            if (lane < nwarps)
            {
                acc[k].s = smem[(k * 32 + lane) * 2 + 0];
                acc[k].c = smem[(k * 32 + lane) * 2 + 1];
            }
            else
                acc[k].zero();
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
            {
                const double os = __shfl_down_sync(0xffffffffu, acc[k].s, off);
                const double oc = __shfl_down_sync(0xffffffffu, acc[k].c, off);
                if (lane < off) acc[k].merge(os, oc);
            }
        }
    }
}

} // namespace mwsep

#endif
