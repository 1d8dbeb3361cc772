/*
 * milkyway_separation_gb300_test.h -- test and diagnostic entry points of
 * libmwsep_gb300.so.
 *
 * These are exported by the same library as the product C ABI
 * (milkyway_separation_gb300.h) but are not part of it: they exist so the
 * library's tests can check a debug build's device index checks, the error
 * bounds of the double-float primitives and the launch model behind a
 * default tile shape.  None has a counterpart in the reference.  A client of
 * the evaluator needs none of them.
 */
#ifndef MILKYWAY_SEPARATION_GB300_TEST_H
#define MILKYWAY_SEPARATION_GB300_TEST_H

#include "milkyway_separation_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Device-side index checks of a debug build (compiled with
 * -DMWSEP_DEVICE_CHECKS=1): *enabled says whether this library has them;
 * *failures counts table indices found out of range since the last call
 * (each was redirected to element 0 instead of being read) and *first is
 * the first one as (tag << 48 | index).  Reading resets the counters.  No
 * reference counterpart. */
int mwsep_device_checks(int device, int* enabled, unsigned long long* failures, unsigned long long* first);
/* The double-float primitives of MWSEP_PLAIN_DF evaluated element-wise on
 * `device`, for testing their error bounds: op 0 2^x, 1 sqrt(x), 2 x / y,
 * 3 x * y, 4 x + y, 5 x y^2 + z, 6 log2(x); ops 10-16 the same through the packed
 * versions the integral kernel uses (elements taken two at a time).  Inputs
 * are doubles (split into FP32 pairs on the device), outputs the pairs'
 * values as doubles; host arrays of n elements (y and z unused by the ops
 * that do not take them), synchronous.  Ops 20 e^x and 21 1/x are the
 * FP64 integral kernel's own table-driven exponential and Newton-Raphson
 * reciprocal, in plain FP64. */
int mwsep_df_eval(int device, int op, int n, const double* x, const double* y, const double* z, double* out);
/* The compensated likelihood's log10 sum (a mantissa product and an exponent
 * sum, log10 taken once) over host values x[0..n) on `device`, in one block
 * with the likelihood kernels' fixed-order combination: *out = sum of
 * log10(x[i]) with log10's semantics per term (0 gives -inf, a negative or
 * NaN term NaN, +inf +inf).  Synchronous. */
int mwsep_log10_sum_eval(int device, int n, const double* x, double* out);

/* The launch model behind the compensated form's default r-chunk (host only,
 * no device needed; no reference counterpart).  mwsep_model_tile_cost: the
 * modelled time, in lane groups of points, of one warp-tile launch with a
 * fixed share of tiles per warp (warp w of W takes tiles w, w + W, ... in
 * r-chunk-major order, block b on SM b % sms): the largest per-SM sum of tile
 * costs, a tile costing ceil(k_chunk' * convolve / group) + prologue for its
 * chunk's k_chunk' bins; -1 on invalid input.  mwsep_model_kchunk: the chunk
 * of least modelled time for a wedge of mu_steps x nu_steps x r_steps cells
 * (the choice the library makes for MWSEP_MIXED_F32), and its cost. */
double mwsep_model_tile_cost(int r_steps, int convolve, int group, long long tiles_per_chunk, int k_chunk, int sms,
                             int blocks_per_sm, int warps_per_block, double prologue);
int mwsep_model_kchunk(int r_steps, int convolve, int n_streams, long long mu_steps, long long nu_steps, int sms,
                       int blocks_per_sm, int* k_chunk, double* cost);

#ifdef __cplusplus
}
#endif

#endif /* MILKYWAY_SEPARATION_GB300_TEST_H */
