"""The allocation-free entry point, mwsep_area_integrals_noalloc.

It exists for callers that cannot let a library allocate device memory (all
memory handed to their own pool, hot paths where cudaMalloc would
synchronise the device, loops that must not fail on allocation).  Here the
caller's buffers are torch tensors; the entry point is called through the C
ABI twice in a row (different parameter vectors, so the second call runs on
the scratch array the first one left behind) and each result is compared
with the context entry point (mwsep_ctx_evaluate, plain FP64) at the FP64
tolerance of the other parity tests.  Collected last on purpose.
"""
import ctypes as C
import math

import numpy as np
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu

REL_INT_F64 = 1e-12
DEG = 180.0 / math.pi


def _density_params(theta, ap, oracle_cls):
    """init_constants for the golden cases' layout (alpha = delta = 1, q and
    r0 optimised, then per stream weight, mu, r, theta, phi, sigma)."""
    from milkywayathome_client_gb300 import native as N
    s = ap.struct
    p = N.mwsep_density_params()
    p.alpha, p.q, p.r0, p.delta = 1.0, theta[0], theta[1], 1.0
    p.aux_bg_profile = 0
    p.number_streams = s.number_streams
    for i in range(s.number_streams):
        w, mu, r, th, ph, sig = theta[2 + 6 * i: 8 + 6 * i]
        l, b = oracle_cls.gc_to_lb(s.wedge, mu, 0.0)
        c = oracle_cls.lbr_to_xyz(l, b, r)
        p.stream_sigma[i] = sig
        for k in range(3):
            p.stream_c[i][k] = c[k]
        p.stream_a[i][0] = math.sin(th) * math.cos(ph)
        p.stream_a[i][1] = math.sin(th) * math.sin(ph)
        p.stream_a[i][2] = math.cos(th)
    return p


@pytest.fixture(scope="module")
def problem(built_library, oracle_built):
    import torch
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case("three_streams")
    ap = mw.AstronomyParameters.read(pf)
    assert ap.number_integrals == 1 and ap.struct.sgr_coordinates == 0
    o = oracle_built.Oracle(pf, sf)
    M, NU, R = o.area_dims(0)
    Cv = ap.convolve
    irv, reff, rp, qw = np.zeros(R), np.zeros(R), np.zeros(R * Cv), np.zeros(R * Cv)
    ids, nus = np.zeros(NU), np.zeros(NU)
    D = C.POINTER(C.c_double)
    o.lib().so_r_tables(o._h, 0, *(a.ctypes.data_as(D) for a in (irv, reff, rp, qw, ids, nus)))
    lb = o.cell_lb(0).reshape(-1, 2)
    geom = np.stack([np.sin(lb[:, 1] / DEG), np.cos(lb[:, 1] / DEG), np.sin(lb[:, 0] / DEG),
                     np.cos(lb[:, 0] / DEG)], axis=1)
    dev = torch.device("cuda:0")
    bufs = {k: torch.tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev)
            for k, v in dict(geom=geom, r_point=rp, qw=qw, reff=reff, irv=irv, ids=ids).items()}
    from milkywayathome_client_gb300 import native as N
    t = N.mwsep_area_tables()
    t.mu_steps, t.nu_steps, t.r_steps, t.convolve = M, NU, R, Cv
    t.geom, t.r_point, t.qw_r3_N = bufs["geom"].data_ptr(), bufs["r_point"].data_ptr(), bufs["qw"].data_ptr()
    t.r_in_mag = t.r_in_mag2 = None
    t.reff_xr_rp3, t.irv, t.ids = bufs["reff"].data_ptr(), bufs["irv"].data_ptr(), bufs["ids"].data_ptr()
    sp = mw.StarPoints.read(sf)
    return {"ap": ap, "sp": sp, "g": g, "tables": t, "bufs": bufs, "oracle": oracle_built.Oracle,
            "S": ap.number_streams}


def _noalloc(problem, theta):
    import torch
    from milkywayathome_client_gb300 import native as N
    S = problem["S"]
    out = torch.full((1 + S,), float("nan"), dtype=torch.float64, device="cuda:0")
    p = _density_params(theta, problem["ap"], problem["oracle"])
    stream = torch.cuda.current_stream().cuda_stream
    rc = N.lib().mwsep_area_integrals_noalloc(C.byref(problem["tables"]), C.byref(p), out.data_ptr(),
                                              C.c_void_p(stream))
    assert rc == N.MWSEP_OK, N.lib().mwsep_status_string(rc)
    torch.cuda.synchronize()
    return out.cpu().numpy().tolist()


def test_noalloc_matches_context_entry_two_calls(problem):
    import milkywayathome_client_gb300 as mw
    base = np.asarray(problem["g"]["theta"])
    thetas = [base, base * (1.0 + 0.01 * np.sin(np.arange(base.size)))]
    with mw.Context(0) as ctx:
        ctx.set_problem(problem["ap"])
        ctx.set_stars(problem["sp"])
        want = [ctx.evaluate(t, mw.MWSEP_PLAIN_F64).area_integrals[0] for t in thetas]
    got = [_noalloc(problem, t) for t in thetas]  # two calls in a row on the shared array
    for gv, wv in zip(got, want):
        for x, y in zip(gv, wv):
            assert abs(x - y) <= REL_INT_F64 * abs(y), (x, y)
    assert got[0] != got[1]
    # and the first parameter vector against the reference's own integrals
    for x, y in zip(got[0], [problem["g"]["background_integral"]] + problem["g"]["stream_integrals"]):
        assert abs(x - y) <= REL_INT_F64 * abs(y), (x, y)


def test_noalloc_rejects_sizes_beyond_the_array(problem):
    from milkywayathome_client_gb300 import native as N
    p = _density_params(problem["g"]["theta"], problem["ap"], problem["oracle"])
    p.number_streams = N.MWSEP_MAX_STREAMS + 1
    rc = N.lib().mwsep_area_integrals_noalloc(C.byref(problem["tables"]), C.byref(p), C.c_void_p(1), None)
    assert rc == N.MWSEP_ERR_UNSUPPORTED
    assert N.lib().mwsep_area_integrals_noalloc(None, C.byref(p), None, None) == N.MWSEP_ERR_ARG
