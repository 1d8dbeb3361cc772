"""GPU parity: the CUDA path against the reference's own outputs (golden
fixtures made by the reference CPU evaluator, tests/golden/make_golden.py) and
against the oracle restatement run live.

Tolerances (plain FP64 form): 1e-12 relative on every integral, 1e-12
absolute on the log-likelihood.  Compensated-FP32 form: 1e-7 absolute on the
log-likelihood.
"""
import math
import os

import numpy as np
import pytest

from conftest import golden_cases, load_case

pytestmark = pytest.mark.gpu

REL_INT_F64 = 1e-12
ABS_LOGL_F64 = 1e-12
ABS_LOGL_F32 = 1e-7


def _close_rel(a, b, tol):
    if math.isnan(a) or math.isnan(b):
        return math.isnan(a) and math.isnan(b)
    if b == 0.0:
        return a == 0.0
    return abs(a - b) <= tol * abs(b)


def _close_abs(a, b, tol):
    if math.isnan(a) or math.isnan(b):
        return math.isnan(a) and math.isnan(b)
    return abs(a - b) <= tol


def _setup(ctx, name):
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case(name)
    ap = mw.AstronomyParameters.read(pf)
    sp = mw.StarPoints.read(sf)
    ctx.set_problem(ap)
    ctx.set_stars(sp)
    return ap, sp, g


@pytest.mark.parametrize("name", golden_cases())
def test_plain_f64_matches_reference(gpu_ctx, name):
    import milkywayathome_client_gb300 as mw
    _, _, g = _setup(gpu_ctx, name)
    r = gpu_ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_F64)
    for a, (got_area, want_area) in enumerate(zip(r.area_integrals, g["area_integrals"])):
        for k, (x, y) in enumerate(zip(got_area, want_area)):
            assert _close_rel(x, y, REL_INT_F64), f"area {a} comp {k}: {x!r} vs {y!r}"
    assert _close_rel(r.background_integral, g["background_integral"], REL_INT_F64)
    for x, y in zip(r.stream_integrals, g["stream_integrals"]):
        assert _close_rel(x, y, REL_INT_F64), (x, y)
    assert _close_abs(r.likelihood, g["likelihood"], ABS_LOGL_F64), (r.likelihood, g["likelihood"])
    assert r.num_zero == g["num_zero"]


# The SFU approximations (ex2 / rsqrt / rcp) carry up to ~2^-22 relative
# error per convolution point.  Averaged over a catalogue that is far below
# 1e-7 in log10; a one-star, one-point problem sees it undiluted.
ABS_LOGL_F32_SINGLE_POINT = 5e-7


@pytest.mark.parametrize("name", golden_cases())
def test_mixed_f32_within_1e7(gpu_ctx, name):
    import milkywayathome_client_gb300 as mw
    _, sp, g = _setup(gpu_ctx, name)
    r = gpu_ctx.evaluate(g["theta"], mw.MWSEP_MIXED_F32)
    tol = ABS_LOGL_F32 if sp.number_stars >= 10 else ABS_LOGL_F32_SINGLE_POINT
    assert _close_abs(r.likelihood, g["likelihood"], tol), \
        f"dlogL {r.likelihood - g['likelihood']:.3e} ({r.likelihood!r} vs {g['likelihood']!r})"
    assert r.num_zero == g["num_zero"]


@pytest.mark.parametrize("name", ["basic_1stream", "cut_area", "three_streams"])
def test_evalfunc_dropin(built_library, name):
    """The EvalFunc entry fills EVALUATION_STATE like cpu_evaluate."""
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case(name)
    ap = mw.AstronomyParameters.read(pf)
    sp = mw.StarPoints.read(sf)
    es = mw.EvaluationState(ap, sp)
    v = mw.evaluate(g["theta"], ap, es, sp)
    assert _close_abs(v - 3.0, g["likelihood"], ABS_LOGL_F64)
    assert _close_rel(es.background_integral, g["background_integral"], REL_INT_F64)
    for x, y in zip(es.stream_integrals, g["stream_integrals"]):
        assert _close_rel(x, y, REL_INT_F64)
    for got_area, want_area in zip(es.area_integrals, g["area_integrals"]):
        for x, y in zip(got_area, want_area):
            assert _close_rel(x, y, REL_INT_F64)
    assert _close_rel(es.prob_sum, g["prob_sum"], 1e-12)
    # theta was applied to the struct, as set_astronomy_parameters does
    np.testing.assert_array_equal(ap.search_parameters(), np.asarray(g["theta"]))
    vm = mw.evaluate_mixed(g["theta"], ap, es, sp)
    assert abs((vm - 3.0) - g["likelihood"]) <= ABS_LOGL_F32
    # the double-float EvalFunc: the plain form's bounds, the same state filled
    es2 = mw.EvaluationState(ap, sp)
    vd = mw.evaluate_df(g["theta"], ap, es2, sp)
    assert _close_abs(vd - 3.0, g["likelihood"], ABS_LOGL_F64)
    assert _close_rel(es2.background_integral, g["background_integral"], REL_INT_F64)
    for x, y in zip(es2.stream_integrals, g["stream_integrals"]):
        assert _close_rel(x, y, REL_INT_F64)
    assert _close_rel(es2.prob_sum, g["prob_sum"], 1e-12)


def test_evalfunc_alternating_catalogues(gpu_ctx):
    """The EvalFunc entries upload each call's catalogue on a side stream
    while the integral runs: alternating two problems whose catalogues
    differ in size and content, every call in every form gives the same bits
    as the context API, which uploads synchronously."""
    import milkywayathome_client_gb300 as mw
    cases = []
    for name in ("three_streams", "basic_1stream"):
        pf, sf, g = load_case(name)
        ap, sp = mw.AstronomyParameters.read(pf), mw.StarPoints.read(sf)
        gpu_ctx.set_problem(ap)
        gpu_ctx.set_stars(sp)
        want = {p: gpu_ctx.evaluate(g["theta"], p).likelihood for p in (0, 1, 2)}
        cases.append((ap, sp, g, want))
    assert cases[0][1].number_stars != cases[1][1].number_stars
    fns = {0: mw.evaluate, 1: mw.evaluate_mixed, 2: mw.evaluate_df}
    for _ in range(3):
        for ap, sp, g, want in cases:
            for p, fn in fns.items():
                es = mw.EvaluationState(ap, sp)
                assert fn(g["theta"], ap, es, sp) - 3.0 == want[p], (p, want[p])


@pytest.mark.parametrize("name", ["three_streams", "aux_profile", "cut_area", "six_streams", "general_alpha_delta",
                                  "stream_off"])
def test_split_likelihood_equals_fused(gpu_ctx, name, monkeypatch):
    """The compensated likelihood's two launches (per-star densities beside
    the integral, then the epilogue) give the fused kernel's bits, alone and
    in a batch."""
    import milkywayathome_client_gb300 as mw
    _, _, g = _setup(gpu_ctx, name)
    base = np.asarray(g["theta"])
    thetas = [base * (1 + 1e-3 * k) for k in range(3)]
    split = [gpu_ctx.evaluate(t, mw.MWSEP_MIXED_F32) for t in thetas]
    split_b = gpu_ctx.evaluate_batch(thetas, mw.MWSEP_MIXED_F32)
    monkeypatch.setenv("MWSEP_SPLIT_LIKELIHOOD", "0")
    fused = [gpu_ctx.evaluate(t, mw.MWSEP_MIXED_F32) for t in thetas]
    def same(x, y):  # equal bits, or both NaN (stream_off's likelihood is NaN, as the reference's)
        return x == y or (math.isnan(x) and math.isnan(y))
    for a, b, c in zip(split, split_b, fused):
        assert same(a.likelihood, b.likelihood) and same(a.likelihood, c.likelihood)
        assert same(a.background_only_likelihood, c.background_only_likelihood)
        assert all(same(x, y) for x, y in zip(a.stream_only_likelihood, c.stream_only_likelihood))
        assert a.num_zero == c.num_zero


@pytest.mark.parametrize("name", ["three_streams", "cut_area", "aux_profile", "general_alpha_delta", "six_streams"])
def test_tile_counter_integral(gpu_ctx, name, monkeypatch):
    """The compensated integral with tiles handed out by a counter against the
    static schedule (sums in another order: within 1e-12), and a batch cut
    into theta chunks equal to the single evaluations bit for bit (cut_area
    has two areas of different tile counts)."""
    import milkywayathome_client_gb300 as mw
    _, _, g = _setup(gpu_ctx, name)
    base = np.asarray(g["theta"])
    thetas = [base * (1 + 1e-3 * k) for k in range(5)]
    single = [gpu_ctx.evaluate(t, mw.MWSEP_MIXED_F32) for t in thetas]
    monkeypatch.setenv("MWSEP_F32_DYN_CHUNK", "2")
    chunked = gpu_ctx.evaluate_batch(thetas, mw.MWSEP_MIXED_F32)
    monkeypatch.delenv("MWSEP_F32_DYN_CHUNK")
    monkeypatch.setenv("MWSEP_F32_DYNAMIC", "0")
    static = [gpu_ctx.evaluate(t, mw.MWSEP_MIXED_F32) for t in thetas]
    for a, b, c in zip(single, chunked, static):
        assert a.integrals == b.integrals and a.area_integrals == b.area_integrals
        assert a.likelihood == b.likelihood or (math.isnan(a.likelihood) and math.isnan(b.likelihood))
        for x, y in zip(a.integrals, c.integrals):
            assert _close_rel(x, y, 1e-12), (x, y)
        assert _close_abs(a.likelihood, c.likelihood, 1e-12)


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_equals_single_bitwise(gpu_ctx, precision):
    """Each result of a batch is bit-identical to the same theta alone."""
    _, _, g = _setup(gpu_ctx, "three_streams")
    base = np.asarray(g["theta"])
    rng = np.random.default_rng(3)
    thetas = base + rng.normal(0, 0.01, size=(5, base.size)) * np.abs(base)
    batch = gpu_ctx.evaluate_batch(thetas, precision)
    for t, b in zip(thetas, batch):
        s = gpu_ctx.evaluate(t, precision)
        assert s.likelihood == b.likelihood
        assert s.integrals == b.integrals


def test_repeatable_bitwise(gpu_ctx):
    _, _, g = _setup(gpu_ctx, "config0")
    a = gpu_ctx.evaluate(g["theta"], 0)
    b = gpu_ctx.evaluate(g["theta"], 0)
    assert a.likelihood == b.likelihood and a.integrals == b.integrals


@pytest.mark.parametrize("name", ["basic_1stream", "general_alpha_delta", "sgr_coordinates"])
def test_against_live_oracle(gpu_ctx, oracle_built, name):
    """Also compare with the oracle restatement (diagnostics included)."""
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case(name)
    want = oracle_built.Oracle(pf, sf).evaluate(g["theta"])
    _setup(gpu_ctx, name)
    r = gpu_ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_F64)
    assert _close_abs(r.likelihood, want["likelihood"], ABS_LOGL_F64)
    assert _close_abs(r.background_only_likelihood, want["background_only_likelihood"], 1e-12)
    for x, y in zip(r.stream_only_likelihood, want["stream_only_likelihood"]):
        assert _close_abs(x, y, 1e-12)


@pytest.mark.parametrize("flag", [None, "--mixed", "--df"])
def test_c_client_matches_reference(built_library, flag):
    """The C command-line client (worker() on the C ABI) prints the
    reference's result lines with the reference's numbers."""
    import re
    import subprocess
    from milkywayathome_client_gb300 import build
    pf, sf, g = load_case("cut_area")
    mixed = flag == "--mixed"
    cmd = [build.CLIENT_PATH, "-a", pf, "-p", sf] + ([flag] if flag else []) + \
        [repr(float(x)) for x in g["theta"]]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    ll = float(re.search(r"<search_likelihood> (\S+) </search_likelihood>", r.stderr).group(1))
    bg = float(re.search(r"<background_integral> (\S+) </background_integral>", r.stderr).group(1))
    assert abs(ll - g["likelihood"]) <= (ABS_LOGL_F32 if mixed else ABS_LOGL_F64)
    if not mixed:
        # printed with %.20lf: compare at the printed precision
        assert abs(bg - g["background_integral"]) <= max(1e-12 * abs(g["background_integral"]), 1e-20)


@pytest.mark.parametrize("name", ["three_streams", "cut_area"])
def test_q_zero_background_integral(gpu_ctx, oracle_built, name):
    """q == 0: every cell's background is -1 times its volume, no density
    (cpu/evaluation_optimized.c:213-216).  Only the background integral is
    comparable (the reference's stream terms then read stale coordinates)."""
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case(name)
    ap = mw.AstronomyParameters.read(pf)
    theta = list(g["theta"])
    assert ap.struct.background_optimize[1]  # q is theta[0] in these cases
    theta[0] = 0.0
    _setup(gpu_ctx, name)
    want = oracle_built.Oracle(pf, sf).integrals(theta)[0][0]
    r64 = gpu_ctx.evaluate(theta, mw.MWSEP_PLAIN_F64)
    r32 = gpu_ctx.evaluate(theta, mw.MWSEP_MIXED_F32)
    rdf = gpu_ctx.evaluate(theta, mw.MWSEP_PLAIN_DF)
    assert _close_rel(r64.background_integral, want, REL_INT_F64), (r64.background_integral, want)
    assert _close_rel(rdf.background_integral, want, REL_INT_F64), (rdf.background_integral, want)
    for x, y in zip(rdf.stream_integrals, r64.stream_integrals):  # same (current-point) stream terms
        assert _close_rel(x, y, REL_INT_F64), (x, y)
    # the compensated form sums the volumes rounded to FP32 once each
    assert _close_rel(r32.background_integral, want, 1e-6), (r32.background_integral, want)


@pytest.mark.parametrize("mu,sigma", [(150.0, 1.0), (200.0, 1.0), (250.0, 0.5), (340.0, 0.5)])
def test_compensated_far_stream(gpu_ctx, mu, sigma):
    """A narrow stream moved far from the wedge (integrals down to 1e-120,
    every density below FP32 range): the compensated form shifts each
    stream's exponents per tile and per star, so its integrals keep their
    FP64 magnitude and the log-likelihood stays within 1e-7 of the plain
    form (without the shift: a zero integral and a NaN likelihood).  The
    engine path as well."""
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case("three_streams")
    _setup(gpu_ctx, "three_streams")
    theta = np.asarray(g["theta"], dtype=np.float64).copy()
    theta[3] = mu     # stream 1: mu (degrees)
    theta[7] = sigma  # stream 1: sigma
    a = gpu_ctx.evaluate(theta, mw.MWSEP_PLAIN_F64)
    b = gpu_ctx.evaluate(theta, mw.MWSEP_MIXED_F32)
    for x, y in zip(b.integrals, a.integrals):
        assert abs(x - y) <= 2e-6 * abs(y), (x, y)
    assert abs(b.likelihood - a.likelihood) <= ABS_LOGL_F32, (b.likelihood, a.likelihood)
    with mw.Context(0) as ctx:
        wid = ctx.add_wedge(mw.AstronomyParameters.read(pf), mw.StarPoints.read(sf))
        e = ctx.evaluate_requests([(wid, theta)], mw.MWSEP_MIXED_F32)[0]
    assert abs(e.likelihood - a.likelihood) <= ABS_LOGL_F32, (e.likelihood, a.likelihood)


def test_compensated_thread_items():
    """The compensated form's thread-item kernels (one column and r-run per
    thread, MWSEP_F32_WARP_TILES=0) against the reference's goldens within
    1e-7 on the log-likelihood, a far stream included (a fresh process: the
    switch is read when a wedge's launch shape is chosen)."""
    import subprocess
    import sys
    import textwrap
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = textwrap.dedent(f"""
        import sys, json, math
        sys.path.insert(0, {root!r}); sys.path.insert(0, {os.path.join(root, "tests")!r})
        import numpy as np
        from conftest import load_case
        import milkywayathome_client_gb300 as mw
        worst = 0.0
        with mw.Context(0) as ctx:
            for name in ("basic_1stream", "three_streams", "cut_area", "aux_profile", "general_alpha_delta"):
                pf, sf, g = load_case(name)
                ctx.set_problem(mw.AstronomyParameters.read(pf)); ctx.set_stars(mw.StarPoints.read(sf))
                r = ctx.evaluate(g["theta"], mw.MWSEP_MIXED_F32)
                worst = max(worst, abs(r.likelihood - g["likelihood"]))
            pf, sf, g = load_case("three_streams")
            ctx.set_problem(mw.AstronomyParameters.read(pf)); ctx.set_stars(mw.StarPoints.read(sf))
            th = np.asarray(g["theta"], float); th[3] = 200.0; th[7] = 1.0
            a = ctx.evaluate(th, mw.MWSEP_PLAIN_F64); b = ctx.evaluate(th, mw.MWSEP_MIXED_F32)
            far = abs(a.likelihood - b.likelihood)
            rel = abs(b.integrals[2] - a.integrals[2]) / a.integrals[2]
        print(json.dumps({{"worst": worst, "far": far, "rel": rel}}))
    """)
    env = dict(os.environ, MWSEP_F32_WARP_TILES="0")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr
    import json
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["worst"] <= ABS_LOGL_F32, res
    assert res["far"] <= ABS_LOGL_F32 and res["rel"] <= 2e-6, res
