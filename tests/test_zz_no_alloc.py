"""The allocation-free entry point, mwsep_area_integrals_noalloc.

It exists for callers that cannot let a library allocate device memory (all
memory handed to their own pool, hot paths where cudaMalloc would
synchronise the device, loops that must not fail on allocation).  Here the
caller's buffers are torch tensors; the entry point is called through the C
ABI twice in a row (different parameter vectors, so the second call runs on
the scratch array the first one left behind) and each result is compared
with the context entry point (mwsep_ctx_evaluate, plain FP64) at the FP64
tolerance of the other parity tests, over background forms (alpha = delta =
1, the aux profile, general alpha/delta) and stream counts (3 and 6), and on
rank slices of an area against the reference's own sliced integrals.
Collected last on purpose.
"""
import ctypes as C
import json
import math
import os

import numpy as np
import pytest

from conftest import CASES, load_case

pytestmark = pytest.mark.gpu

REL_INT_F64 = 1e-12
DEG = 180.0 / math.pi


def _density_params(theta, ap, oracle_cls):
    """init_constants (cpu/evaluation_optimized.c:54-133) for theta, read
    back from the problem struct after set_astronomy_parameters."""
    from milkywayathome_client_gb300 import native as N
    ap.set_parameters(theta)
    s = ap.struct
    bg = [s.background_parameters[i] for i in range(s.number_background_parameters)]
    p = N.mwsep_density_params()
    p.alpha, p.q, p.r0, p.delta = bg[0], bg[1], bg[2], bg[3]
    p.aux_bg_profile = s.aux_bg_profile
    if s.aux_bg_profile:
        p.bg_a, p.bg_b, p.bg_c = bg[4], bg[5], bg[6]
    p.number_streams = s.number_streams
    for i in range(s.number_streams):
        mu, r, th, ph, sig = (s.stream_parameters[i][k] for k in range(5))
        l, b = oracle_cls.gc_to_lb(s.wedge, mu, 0.0)
        c = oracle_cls.lbr_to_xyz(l, b, r)
        p.stream_sigma[i] = sig
        for k in range(3):
            p.stream_c[i][k] = c[k]
        p.stream_a[i][0] = math.sin(th) * math.cos(ph)
        p.stream_a[i][1] = math.sin(th) * math.sin(ph)
        p.stream_a[i][2] = math.cos(th)
    return p


def _problem(name, oracle_built):
    import torch
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import native as N
    pf, sf, g = load_case(name)
    ap = mw.AstronomyParameters.read(pf)
    assert ap.struct.sgr_coordinates == 0
    o = oracle_built.Oracle(pf, sf)
    M, NU, R = o.area_dims(0)
    Cv = ap.convolve
    irv, reff, rp, qw = np.zeros(R), np.zeros(R), np.zeros(R * Cv), np.zeros(R * Cv)
    gm, gm2 = np.zeros(R * Cv), np.zeros(R * Cv)
    ids, nus = np.zeros(NU), np.zeros(NU)
    D = C.POINTER(C.c_double)
    o.lib().so_r_tables(o._h, 0, *(a.ctypes.data_as(D) for a in (irv, reff, rp, qw, ids, nus)))
    o.lib().so_r_mag_tables(o._h, 0, gm.ctypes.data_as(D), gm2.ctypes.data_as(D))
    lb = o.cell_lb(0).reshape(-1, 2)
    geom = np.stack([np.sin(lb[:, 1] / DEG), np.cos(lb[:, 1] / DEG), np.sin(lb[:, 0] / DEG),
                     np.cos(lb[:, 0] / DEG)], axis=1)
    dev = torch.device("cuda:0")
    bufs = {k: torch.tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev)
            for k, v in dict(geom=geom, r_point=rp, qw=qw, gm=gm, gm2=gm2, reff=reff, irv=irv, ids=ids).items()}
    t = N.mwsep_area_tables()
    t.mu_steps, t.nu_steps, t.r_steps, t.convolve = M, NU, R, Cv
    t.geom, t.r_point, t.qw_r3_N = bufs["geom"].data_ptr(), bufs["r_point"].data_ptr(), bufs["qw"].data_ptr()
    t.r_in_mag, t.r_in_mag2 = bufs["gm"].data_ptr(), bufs["gm2"].data_ptr()
    t.reff_xr_rp3, t.irv, t.ids = bufs["reff"].data_ptr(), bufs["irv"].data_ptr(), bufs["ids"].data_ptr()
    t.min_calculation, t.max_calculation = 0, M * NU * R
    sp = mw.StarPoints.read(sf)
    return {"pf": pf, "sf": sf, "ap": ap, "sp": sp, "g": g, "tables": t, "bufs": bufs,
            "oracle": oracle_built.Oracle, "S": ap.number_streams, "cells": M * NU * R}


@pytest.fixture(scope="module", params=["three_streams", "aux_profile", "general_alpha_delta", "six_streams"])
def problem(request, built_library, oracle_built):
    return _problem(request.param, oracle_built)


def _noalloc(problem, theta, tables=None):
    import torch
    from milkywayathome_client_gb300 import native as N
    S = problem["S"]
    out = torch.full((1 + S,), float("nan"), dtype=torch.float64, device="cuda:0")
    p = _density_params(theta, problem["ap"], problem["oracle"])
    stream = torch.cuda.current_stream().cuda_stream
    rc = N.lib().mwsep_area_integrals_noalloc(C.byref(tables or problem["tables"]), C.byref(p), out.data_ptr(),
                                              C.c_void_p(stream))
    assert rc == N.MWSEP_OK, N.lib().mwsep_status_string(rc)
    torch.cuda.synchronize()
    return out.cpu().numpy().tolist()


def test_noalloc_matches_context_entry_two_calls(problem):
    import milkywayathome_client_gb300 as mw
    base = np.asarray(problem["g"]["theta"])
    thetas = [base, base * (1.0 + 0.01 * np.sin(np.arange(base.size)))]
    with mw.Context(0) as ctx:
        ctx.set_problem(mw.AstronomyParameters.read(problem["pf"]))
        ctx.set_stars(problem["sp"])
        want = [ctx.evaluate(t, mw.MWSEP_PLAIN_F64).area_integrals[0] for t in thetas]
    got = [_noalloc(problem, t) for t in thetas]  # two calls in a row on the shared array
    for gv, wv in zip(got, want):
        for x, y in zip(gv, wv):
            assert abs(x - y) <= REL_INT_F64 * abs(y), (x, y)
    assert got[0] != got[1]
    # and the first parameter vector against the reference's own area integrals
    for x, y in zip(got[0], problem["g"]["area_integrals"][0]):
        assert abs(x - y) <= REL_INT_F64 * abs(y), (x, y)


def test_noalloc_slices_match_reference(built_library, oracle_built):
    """Each rank's cells [min_calculation, max_calculation) of config0's area
    against the reference's sliced evaluation, two calls per rank."""
    pr = _problem("config0", oracle_built)
    with open(os.path.join(CASES, "config0", "golden_slices.json")) as f:
        slices = json.load(f)
    t = pr["tables"]
    total = pr["cells"]
    for g in slices:
        n = g["nranks"]
        t.min_calculation = int(total * (g["rank"] / n))
        t.max_calculation = int(total * ((g["rank"] + 1) / n))
        for _ in range(2):
            got = _noalloc(pr, g["theta"], t)
            for x, y in zip(got, g["area_integrals"][0]):
                assert abs(x - y) <= REL_INT_F64 * abs(y), (g["rank"], x, y)


def test_noalloc_rejects_sizes_beyond_the_array(problem):
    """Rejected requests return before any launch: the output buffer keeps
    its NaNs."""
    import torch
    from milkywayathome_client_gb300 import native as N
    out = torch.full((1 + N.MWSEP_MAX_STREAMS + 1,), float("nan"), dtype=torch.float64, device="cuda:0")
    t = problem["tables"]

    def call(p, tables=t):
        rc = N.lib().mwsep_area_integrals_noalloc(C.byref(tables), C.byref(p), out.data_ptr(), None)
        torch.cuda.synchronize()
        return rc

    p = _density_params(problem["g"]["theta"], problem["ap"], problem["oracle"])
    p.number_streams = N.MWSEP_MAX_STREAMS + 1
    assert call(p) == N.MWSEP_ERR_UNSUPPORTED
    p = _density_params(problem["g"]["theta"], problem["ap"], problem["oracle"])
    big = N.mwsep_area_tables.from_buffer_copy(t)
    big.convolve = N.MWSEP_MAX_CONVOLVE + 1
    assert call(p, big) == N.MWSEP_ERR_UNSUPPORTED
    neg = N.mwsep_area_tables.from_buffer_copy(t)
    neg.min_calculation = -1
    assert call(p, neg) == N.MWSEP_ERR_ARG
    aux = N.mwsep_area_tables.from_buffer_copy(t)
    aux.r_in_mag = None
    p.aux_bg_profile = 1
    assert call(p, aux) == N.MWSEP_ERR_ARG
    assert N.lib().mwsep_area_integrals_noalloc(None, C.byref(p), None, None) == N.MWSEP_ERR_ARG
    assert bool(torch.isnan(out).all()), "a rejected call wrote its output"
