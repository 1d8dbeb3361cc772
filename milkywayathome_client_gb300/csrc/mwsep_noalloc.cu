/* mwsep_noalloc.cu -- the allocation-free entry point.
 *
 * Some callers cannot let a library call cudaMalloc: programs that hand all
 * device memory to their own pool or arena up front, drivers that must not
 * allocate on their hot path because cudaMalloc can synchronise the device
 * and stall work queued on other streams, and real-time loops that may not
 * fail on allocation once running.  mwsep_area_integrals_noalloc serves them:
 * the caller owns every input and output buffer, and the only device memory
 * the call uses besides those is the fixed array below, which the library
 * image carries.
 *
 * The array is file-scope device memory of MWSEP_NOALLOC_SCRATCH_BYTES
 * bytes.  It is part of the loaded module, so every GPU that loads this
 * library holds it until the process exits.  Host code must not take the
 * array's name as a device address (on the host it names a shadow variable):
 * the device address comes from cudaGetSymbolAddress, fetched once per device
 * with that device current, on the first call made on that device.
 *
 * Layout of the array for one call:
 *   [0, 1 KiB)      the evaluation constants (written by a kernel each call)
 *   [1 KiB, 2 KiB)  the per-area integrals the reduction also writes
 *   [2 KiB, end)    per-block compensated partial sums, grid x (1+S) x 16 B
 * Every byte a kernel reads is written earlier in the same call, so nothing
 * has to be cleared between calls; the array simply keeps the last call's
 * contents.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>

#include "milkyway_separation_gb300.h"
#include "mwsep_internal.h"
#include "mwsep_status.h"

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[MWSEP_NOALLOC_SCRATCH_BYTES];

constexpr size_t kThetaOffset = 0;
constexpr size_t kAreasOffset = 1024;
constexpr size_t kPartialsOffset = 2048;
constexpr int kBlock = 256;
constexpr int kMaxDevices = 64;

/* The layout holds for every accepted request: the constants fit their
 * slot, one area's 1 + S results fit theirs, and the stream limit the call
 * accepts is one the kernels are specialised for (blocks_per_sm is indexed
 * by it). */
static_assert(sizeof(mwsep_theta_consts) <= kAreasOffset - kThetaOffset, "constants overlap the area results");
static_assert((1 + MWSEP_MAX_STREAMS) * sizeof(double) <= kPartialsOffset - kAreasOffset,
              "area results overlap the partial sums");
static_assert(MWSEP_MAX_STREAMS <= MWSEP_KMAX_STREAMS, "stream limit beyond the kernels' specialisation");
static_assert(kPartialsOffset + (1 + MWSEP_MAX_STREAMS) * sizeof(double2) <= MWSEP_NOALLOC_SCRATCH_BYTES,
              "no room for one block's partial sums");

/* A failed launch: its name and CUDA error under MWSEP_DEBUG, then the
 * status (the CUDA error itself is cleared by cudaGetLastError). */
int launch_failed(const char* what, cudaError_t e)
{
    if (getenv("MWSEP_DEBUG")) fprintf(stderr, "mwsep_area_integrals_noalloc: %s failed: %s\n", what, cudaGetErrorString(e));
    return mwsep_fail(MWSEP_ERR_CUDA);
}

struct DeviceSetup
{
    unsigned char* scratch = nullptr; /* device address of g_noalloc_scratch */
    int sm_count = 0;
    int blocks_per_sm[MWSEP_KMAX_STREAMS + 1] = {};
};

std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

/* Writes the evaluation constants into the scratch array (no host staging). */
__global__ void store_theta_kernel(const mwsep_theta_consts th, mwsep_theta_consts* dst)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = th;
}

int setup_device(int dev, DeviceSetup*& out)
{
    if (dev < 0 || dev >= kMaxDevices) return MWSEP_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup& d = g_setup[dev];
    if (!d.scratch)
    {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
        {
            cudaGetLastError();
            return MWSEP_ERR_CUDA;
        }
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        {
            cudaGetLastError();
            return MWSEP_ERR_CUDA;
        }
        for (int s = 0; s <= MWSEP_KMAX_STREAMS; ++s) d.blocks_per_sm[s] = mwsep_integral_f64_blocks_per_sm(s, kBlock);
        d.sm_count = sms;
        d.scratch = (unsigned char*)p;
    }
    out = &d;
    return MWSEP_OK;
}

} // namespace

extern "C" int mwsep_area_integrals_noalloc(const mwsep_area_tables* t, const mwsep_density_params* p,
                                            double* d_integrals, void* stream)
{
    if (!t || !p || !d_integrals) return mwsep_fail(MWSEP_ERR_ARG);
    if (!t->geom || !t->r_point || !t->qw_r3_N || !t->reff_xr_rp3 || !t->irv || !t->ids)
        return mwsep_fail(MWSEP_ERR_ARG);
    if (t->mu_steps < 1 || t->nu_steps < 1 || t->r_steps < 1 || t->convolve < 1) return mwsep_fail(MWSEP_ERR_ARG);
    if (p->aux_bg_profile != 0 && p->aux_bg_profile != 1) return mwsep_fail(MWSEP_ERR_ARG);
    if (p->aux_bg_profile == 1 && (!t->r_in_mag || !t->r_in_mag2)) return mwsep_fail(MWSEP_ERR_ARG);
    /* sizes beyond what the fixed array was laid out for */
    if (p->number_streams < 0 || p->number_streams > MWSEP_MAX_STREAMS) return mwsep_fail(MWSEP_ERR_UNSUPPORTED);
    if (t->convolve > MWSEP_MAX_CONVOLVE) return mwsep_fail(MWSEP_ERR_UNSUPPORTED);
    if ((long long)t->mu_steps * t->nu_steps > (1LL << 30)) return mwsep_fail(MWSEP_ERR_UNSUPPORTED);
    const long long cols = (long long)t->mu_steps * t->nu_steps;
    long long cell_begin, cell_end;
    if (!mwsep::effective_slice(t->min_calculation, t->max_calculation, cols * t->r_steps, cell_begin, cell_end))
        return mwsep_fail(MWSEP_ERR_ARG);

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
    {
        cudaGetLastError();
        return mwsep_fail(MWSEP_ERR_CUDA);
    }
    DeviceSetup* d = nullptr;
    int rc = setup_device(dev, d);
    if (rc) return mwsep_fail(rc);

    const int S = p->number_streams;
    const int ncomp = 1 + S;
    const size_t per_block = (size_t)ncomp * sizeof(double2);
    const long long grid_cap = (long long)((MWSEP_NOALLOC_SCRATCH_BYTES - kPartialsOffset) / per_block);

    /* evaluation constants, as init_constants (cpu/evaluation_optimized.c:54-133)
     * leaves them */
    mwsep_theta_consts th;
    memset(&th, 0, sizeof(th));
    th.alpha = p->alpha;
    th.q = p->q;
    th.r0 = p->r0;
    th.delta = p->delta;
    th.aux = p->aux_bg_profile;
    if (th.aux)
    {
        th.bg_a = p->bg_a;
        th.bg_b = p->bg_b;
        th.bg_c = p->bg_c;
    }
    th.alpha_delta3 = 3 - th.alpha + th.delta;
    th.bg_mode = (th.q == 0) ? 2 : ((th.alpha == 1 && th.delta == 1) ? 0 : 1);
    th.n_streams = S;
    for (int s = 0; s < S; ++s)
    {
        const double sigma = p->stream_sigma[s];
        th.sigma_sq2[s] = 2.0 * sigma * sigma;
        th.stream_on[s] = !(sigma > -0.0001 && sigma < 0.0001);
        for (int k = 0; k < 3; ++k)
        {
            th.a[s][k] = p->stream_a[s][k];
            th.c[s][k] = p->stream_c[s][k];
        }
    }

    /* launch shape: a persistent grid that fits the fixed partial-sum area,
     * items of ~48 per thread as the context path picks them */
    const int per_sm = d->blocks_per_sm[S];
    long long grid = std::min<long long>((long long)d->sm_count * per_sm, grid_cap);
    const long long want_items = grid * kBlock * 48;
    long long chunks = std::max<long long>(1, std::min<long long>((want_items + cols - 1) / cols, t->r_steps));
    const int k_chunk = (int)((t->r_steps + chunks - 1) / chunks);

    mwsep_area_dev a;
    memset(&a, 0, sizeof(a));
    a.mu_steps = t->mu_steps;
    a.nu_steps = t->nu_steps;
    a.r_steps = t->r_steps;
    a.convolve = t->convolve;
    a.n_cols = (int)cols;
    mwsep::set_slice(a, cell_begin, cell_end);
    mwsep::set_chunking(a, k_chunk, 0); /* the slice's boxes and item count */
    grid = std::max<long long>(1, std::min<long long>(grid, (a.n_items + kBlock - 1) / kBlock));
    if (kPartialsOffset + (size_t)grid * per_block > MWSEP_NOALLOC_SCRATCH_BYTES)
        return mwsep_fail(MWSEP_ERR_UNSUPPORTED);
    a.geom = t->geom;
    a.r_point = t->r_point;
    a.qw = t->qw_r3_N;
    /* read only by the aux profile; any valid pointer otherwise */
    a.r_in_mag = t->r_in_mag ? t->r_in_mag : t->r_point;
    a.r_in_mag2 = t->r_in_mag2 ? t->r_in_mag2 : t->r_point;
    a.reff = t->reff_xr_rp3;
    a.irv = t->irv;
    a.ids = t->ids;

    mwsep_theta_consts* d_th = (mwsep_theta_consts*)(d->scratch + kThetaOffset);
    double* d_areas = (double*)(d->scratch + kAreasOffset);
    double2* d_part = (double2*)(d->scratch + kPartialsOffset);
    cudaStream_t st = (cudaStream_t)stream;

    mwsep_launch_shape sh;
    memset(&sh, 0, sizeof(sh));
    sh.n_theta = 1;
    sh.n_streams = S;
    sh.n_areas = 1;
    sh.area_index = 0;
    sh.block = kBlock;
    sh.grid = (int)grid;

    store_theta_kernel<<<1, 32, 0, st>>>(th, d_th);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return launch_failed("the constants' store", e);
    e = (cudaError_t)mwsep_launch_integral_f64(&a, d_th, &sh, d_part, st);
    if (e != cudaSuccess) return launch_failed("the integral", e);
    /* one area: the reduction's cut-subtracted result is the area result and
     * goes straight to the caller's buffer */
    e = (cudaError_t)mwsep_launch_reduce_integrals(d_part, &sh, d_areas, d_integrals, st);
    if (e != cudaSuccess) return launch_failed("the reduction", e);
    return MWSEP_OK;
}
