/* Host check of how an integral area's cells are enumerated (no GPU).
 *
 * For seeded grids and slices it compares, cell for cell:
 *   - the cells the reference's calculate_integral visits for an
 *     INTEGRAL_AREA with [min_calculation, max_calculation)
 *     (cpu/evaluation_optimized.c:461-530 with get_steps,
 *     cpu/evaluation_state.c:129-151), restated as a loop here;
 *   - the cells the library's kernels visit: every thread item
 *     (mwsep::item_pos) and every warp tile (mwsep::tile_pos) of the area
 *     view that set_slice / set_chunking build, for several r-chunks.
 * Each cell must be visited exactly once by each enumeration.  Prints
 * "slice harness: ok" and exits 0 on success.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include <vector_types.h>

#include "mwsep_internal.h"

namespace {

unsigned long long g_state = 0x9e3779b97f4a7c15ull;
unsigned long long next_u64()
{
    unsigned long long z = (g_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
long long uniform(long long lo, long long hi) { return lo + (long long)(next_u64() % (unsigned long long)(hi - lo + 1)); }

/* The reference's walk: start at min, step mu -> nu -> r, stop after the
 * cell that brings the count to max. */
std::vector<char> reference_walk(int M, int NU, int R, long long min_calc, long long max_calc)
{
    std::vector<char> seen((size_t)M * NU * R, 0);
    long long current = min_calc;
    int r_step = (int)(current % R);
    int nu_step = (int)((current / R) % NU);
    int mu_step = (int)(current / ((long long)R * NU));
    for (; mu_step < M; mu_step++)
    {
        for (; nu_step < NU; nu_step++)
        {
            for (; r_step < R; r_step++)
            {
                seen[((size_t)mu_step * NU + nu_step) * R + r_step]++;
                current++;
                if (current >= max_calc) break;
            }
            if (current >= max_calc) break;
            r_step = 0;
        }
        if (current >= max_calc) break;
        nu_step = 0;
    }
    return seen;
}

int fail(const char* what, int M, int NU, int R, long long a, long long b, int kc)
{
    fprintf(stderr, "slice harness: %s (grid %d x %d x %d, slice [%lld, %lld), k_chunk %d)\n", what, M, NU, R, a, b,
            kc);
    return 1;
}

int check(int M, int NU, int R, long long min_calc, long long max_calc)
{
    const long long total = (long long)M * NU * R;
    const std::vector<char> want = reference_walk(M, NU, R, min_calc, max_calc);
    long long begin, end;
    if (!mwsep::effective_slice(min_calc, max_calc, total, begin, end))
        return fail("negative start refused", M, NU, R, min_calc, max_calc, 0);
    for (long long i = 0; i < total; ++i)
        if ((want[(size_t)i] != 0) != (i >= begin && i < end))
            return fail("effective range differs from the reference walk", M, NU, R, min_calc, max_calc, 0);
    mwsep_area_dev v;
    memset(&v, 0, sizeof(v));
    v.mu_steps = M;
    v.nu_steps = NU;
    v.r_steps = R;
    v.n_cols = M * NU;
    mwsep::set_slice(v, begin, end);
    const int chunks[] = {1, 2, 3, 7, R};
    for (int kc : chunks)
    {
        for (int warp = 0; warp < 2; ++warp)
        {
            mwsep::set_chunking(v, kc, warp);
            if (v.n_boxes > MWSEP_MAX_BOXES) return fail("too many boxes", M, NU, R, min_calc, max_calc, kc);
            std::vector<char> got((size_t)total, 0);
            for (long long it = 0; it < v.n_items; ++it)
            {
                int mu0, ncols, nu, k0, k1;
                if (warp)
                {
                    const mwsep::TilePos p = mwsep::tile_pos(v, it);
                    mu0 = p.mu0, ncols = p.ncols, nu = p.nu, k0 = p.k0, k1 = p.k1;
                }
                else
                {
                    const mwsep::ItemPos p = mwsep::item_pos(v, it);
                    if (p.col % NU != p.nu) return fail("item column and nu disagree", M, NU, R, min_calc, max_calc, kc);
                    mu0 = p.col / NU, ncols = 1, nu = p.nu, k0 = p.k0, k1 = p.k1;
                }
                if (ncols < 1 || ncols > mwsep::kTileCols || mu0 < 0 || mu0 + ncols > M || nu < 0 || nu >= NU ||
                    k0 < 0 || k1 > R || k1 <= k0 || k1 - k0 > v.k_chunk)
                    return fail("item outside the grid", M, NU, R, min_calc, max_calc, kc);
                for (int i = mu0; i < mu0 + ncols; ++i)
                    for (int k = k0; k < k1; ++k) got[((size_t)i * NU + nu) * R + k]++;
            }
            for (long long i = 0; i < total; ++i)
                if (got[(size_t)i] != want[(size_t)i])
                    return fail(warp ? "warp tiles visit other cells" : "thread items visit other cells", M, NU, R,
                                min_calc, max_calc, kc);
        }
    }
    return 0;
}

} // namespace

int main()
{
    int cases = 0;
    /* every slice of a few small grids, then seeded slices of larger ones */
    const int small[][3] = {{1, 1, 1}, {1, 1, 5}, {3, 1, 4}, {1, 4, 3}, {3, 4, 5}, {5, 2, 1}, {33, 3, 2}};
    for (const auto& g : small)
    {
        const long long total = (long long)g[0] * g[1] * g[2];
        for (long long a = 0; a <= total; ++a)
            for (long long b = 0; b <= total + 1; ++b)
            {
                if (check(g[0], g[1], g[2], a, b)) return 1;
                ++cases;
            }
    }
    for (int t = 0; t < 400; ++t)
    {
        const int M = (int)uniform(1, 80), NU = (int)uniform(1, 20), R = (int)uniform(1, 30);
        const long long total = (long long)M * NU * R;
        const int nranks = (int)uniform(1, 9);
        const int rank = (int)uniform(0, nranks - 1);
        /* split_astronomy_parameters (cpu/parameters.c:502-522) */
        const long long a = (long long)(total * ((double)rank / (double)nranks));
        const long long b = (long long)(total * ((double)(rank + 1) / (double)nranks));
        if (check(M, NU, R, a, b)) return 1;
        if (check(M, NU, R, uniform(0, total), uniform(0, total + 3))) return 1;
        cases += 2;
    }
    printf("slice harness: ok (%d slices)\n", cases);
    return 0;
}
