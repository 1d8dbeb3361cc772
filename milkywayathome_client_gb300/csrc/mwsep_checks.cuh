/* mwsep_checks.cuh -- device-side index checks of a debug build.
 *
 * Built with -DMWSEP_DEVICE_CHECKS=1, every instrumented table index goes
 * through MWSEP_IDX(i, n, tag): an index outside [0, n) is counted, the first
 * one is recorded as (tag << 48 | index), and the access is redirected to
 * element 0 of the same table, so a bad index is reported instead of read.
 * Without the flag MWSEP_IDX(i, n, tag) is i and costs nothing.
 *
 * Each translation unit with kernels has its own counters (no relocatable
 * device code) and exports a reader; mwsep_device_checks() sums them.
 *
 * Tags: 1 area geometry, 2 area point table (row or point), 3 ids, 4 irv,
 * 5 FP64 r-bin row, 6 reff, 7 star (all of its tables), 10 request,
 * 11 area descriptor, 12 catalogue descriptor.
 */
#ifndef MWSEP_CHECKS_CUH
#define MWSEP_CHECKS_CUH

#include <cuda_runtime.h>

#ifndef MWSEP_DEVICE_CHECKS
#define MWSEP_DEVICE_CHECKS 0
#endif

#if MWSEP_DEVICE_CHECKS
namespace mwsep {
namespace checks {
static __device__ unsigned int g_fail;
static __device__ unsigned long long g_first;

__device__ __forceinline__ long long index(long long i, long long n, int tag)
{
    if (i < 0 || i >= n)
    {
        if (atomicAdd(&g_fail, 1u) == 0u)
            g_first = ((unsigned long long)tag << 48) | ((unsigned long long)i & 0xffffffffffffULL);
        return 0;
    }
    return i;
}

/* This translation unit's counters (and reset them). */
static inline int read_and_reset(unsigned long long* fail, unsigned long long* first)
{
    unsigned int n = 0;
    unsigned long long f = 0;
    if (cudaMemcpyFromSymbol(&n, g_fail, sizeof(n)) != cudaSuccess) return 1;
    if (cudaMemcpyFromSymbol(&f, g_first, sizeof(f)) != cudaSuccess) return 1;
    const unsigned int zero = 0;
    const unsigned long long zero64 = 0;
    if (cudaMemcpyToSymbol(g_fail, &zero, sizeof(zero)) != cudaSuccess) return 1;
    if (cudaMemcpyToSymbol(g_first, &zero64, sizeof(zero64)) != cudaSuccess) return 1;
    *fail += n;
    if (!*first && n) *first = f;
    return 0;
}
} // namespace checks
} // namespace mwsep
#define MWSEP_IDX(i, n, tag) ::mwsep::checks::index((long long)(i), (long long)(n), (tag))
#define MWSEP_CHECKS_READER(name)                                                                  \
    extern "C" int name(unsigned long long* fail, unsigned long long* first)                      \
    {                                                                                             \
        return ::mwsep::checks::read_and_reset(fail, first);                                      \
    }
#else
#define MWSEP_IDX(i, n, tag) (i)
#define MWSEP_CHECKS_READER(name)
#endif

#endif
