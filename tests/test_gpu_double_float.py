"""GPU: the double-float form (MWSEP_PLAIN_DF) against the reference's own
outputs at the plain form's tolerances (1e-12 relative on every integral,
1e-12 absolute on the log-likelihood) -- every golden case, the aux profile
included -- against the native FP64 kernel at full size, batch == single,
engine requests and gradients, first use from several threads, the device
memory budget, a batch mixing the background forms, the autotuner, and its
limits (beyond 4 streams the likelihood runs in native FP64).  q = 0 is
checked with the plain form in test_gpu_parity."""
import math
import os

import numpy as np
import pytest

from conftest import golden_cases, load_case

pytestmark = pytest.mark.gpu

REL = 1e-12
ABS_LOGL = 1e-12


def _close_rel(a, b, tol):
    if math.isnan(a) or math.isnan(b):
        return math.isnan(a) and math.isnan(b)
    if b == 0.0:
        return a == 0.0
    return abs(a - b) <= tol * abs(b)


def _setup(ctx, name):
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case(name)
    ctx.set_problem(mw.AstronomyParameters.read(pf))
    ctx.set_stars(mw.StarPoints.read(sf))
    return g


@pytest.mark.parametrize("name", golden_cases())
def test_double_float_matches_reference(gpu_ctx, name):
    import milkywayathome_client_gb300 as mw
    g = _setup(gpu_ctx, name)
    r = gpu_ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_DF)
    for a, (got, want) in enumerate(zip(r.area_integrals, g["area_integrals"])):
        for k, (x, y) in enumerate(zip(got, want)):
            assert _close_rel(x, y, REL), f"area {a} comp {k}: {x!r} vs {y!r}"
    assert _close_rel(r.background_integral, g["background_integral"], REL)
    for x, y in zip(r.stream_integrals, g["stream_integrals"]):
        assert _close_rel(x, y, REL), (x, y)
    if not math.isnan(g["likelihood"]):
        assert abs(r.likelihood - g["likelihood"]) <= ABS_LOGL, (r.likelihood, g["likelihood"])
    assert r.num_zero == g["num_zero"]


def test_double_float_batch_equals_single(gpu_ctx):
    import milkywayathome_client_gb300 as mw
    g = _setup(gpu_ctx, "three_streams")
    base = np.asarray(g["theta"])
    thetas = [base * (1 + 1e-3 * k) for k in range(5)]
    single = [gpu_ctx.evaluate(t, mw.MWSEP_PLAIN_DF) for t in thetas]
    batch = gpu_ctx.evaluate_batch(thetas, mw.MWSEP_PLAIN_DF)
    for a, b in zip(single, batch):
        assert a.likelihood == b.likelihood and a.integrals == b.integrals


def test_double_float_matches_native_fp64_at_full_size(gpu_ctx):
    """Config 0 at full size (80 x 40 x 70 cells, convolve 30)."""
    import milkywayathome_client_gb300 as mw
    g = _setup(gpu_ctx, "config0")
    a = gpu_ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_F64)
    b = gpu_ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_DF)
    for x, y in zip(b.integrals, a.integrals):
        assert _close_rel(x, y, REL), (x, y)
    assert abs(a.likelihood - b.likelihood) <= ABS_LOGL


def test_double_float_limits(gpu_ctx):
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import native as N
    # more than 4 streams: the double-float integral with the FP64 likelihood
    g = _setup(gpu_ctx, "six_streams")
    a = gpu_ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_F64)
    b = gpu_ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_DF)
    assert a.integrals != b.integrals
    for x, y in zip(b.integrals, a.integrals):
        assert _close_rel(x, y, REL), (x, y)
    assert abs(a.likelihood - b.likelihood) <= ABS_LOGL


def test_double_float_autotune():
    """The autotuner times double-float evaluations over candidate r-chunks
    and keeps one; results with the chosen chunk stay within the plain
    form's tolerance of the reference."""
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case("config0")
    with mw.Context(0) as ctx:
        wid = ctx.add_wedge(mw.AstronomyParameters.read(pf), mw.StarPoints.read(sf))
        ms = ctx.autotune(wid, mw.MWSEP_PLAIN_DF)
        assert ms > 0
        kc, _ = ctx.tile_shape(wid, mw.MWSEP_PLAIN_DF)
        assert kc >= 1
        r = ctx.evaluate_requests([(wid, g["theta"])], mw.MWSEP_PLAIN_DF)[0]
        assert abs(r.likelihood - g["likelihood"]) <= ABS_LOGL
        for x, y in zip([r.background_integral] + list(r.stream_integrals),
                        [g["background_integral"]] + list(g["stream_integrals"])):
            assert _close_rel(x, y, REL), (x, y)


def test_double_float_engine_requests():
    """Engine requests in the double-float form over three wedges, in mixed
    order: each result equals the single-wedge evaluation of its wedge bit
    for bit, and stays within the plain form's tolerance of the reference."""
    import milkywayathome_client_gb300 as mw
    names = ["basic_1stream", "three_streams", "four_streams_c120"]
    cases = [load_case(n) for n in names]
    with mw.Context(0) as ctx:
        ids = [ctx.add_wedge(mw.AstronomyParameters.read(pf), mw.StarPoints.read(sf)) for pf, sf, _ in cases]
        reqs = []
        for k in range(3):
            for wid, (_, _, g) in zip(ids, cases):
                reqs.append((wid, np.asarray(g["theta"]) * (1 + 1e-3 * k)))
        reqs = reqs[::-1]
        res = ctx.evaluate_requests(reqs, mw.MWSEP_PLAIN_DF)
    for (wid, th), r in zip(reqs, res):
        pf, sf, g = cases[ids.index(wid)]
        with mw.Context(0) as one:
            one.set_problem(mw.AstronomyParameters.read(pf))
            one.set_stars(mw.StarPoints.read(sf))
            s = one.evaluate(th, mw.MWSEP_PLAIN_DF)
        assert r.integrals == s.integrals and r.likelihood == s.likelihood
        if np.array_equal(th, np.asarray(g["theta"])):
            assert _close_rel(r.background_integral, g["background_integral"], REL)
            assert abs(r.likelihood - g["likelihood"]) <= ABS_LOGL


def test_double_float_gradient_matches_plain(gpu_ctx):
    """Central-difference gradient in the double-float form against the same
    in native FP64: each evaluation agrees to ~1e-14, so the differences
    agree to ~1e-14 / step."""
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case("three_streams")
    with mw.Context(0) as ctx:
        wid = ctx.add_wedge(mw.AstronomyParameters.read(pf), mw.StarPoints.read(sf))
        step = np.full(len(g["theta"]), 1e-3)
        f0a, ga = ctx.gradient(wid, g["theta"], step, mw.MWSEP_PLAIN_F64)
        f0b, gb = ctx.gradient(wid, g["theta"], step, mw.MWSEP_PLAIN_DF)
    assert abs(f0a - f0b) <= ABS_LOGL
    np.testing.assert_allclose(gb, ga, rtol=0, atol=1e-12 / 1e-3)


@pytest.mark.parametrize("mu,sigma", [(200.0, 1.0), (250.0, 0.5), (300.0, 1.0), (340.0, 0.5)])
def test_double_float_far_stream(gpu_ctx, mu, sigma):
    """A narrow stream moved far from the wedge: its terms sit hundreds of
    binary orders below 1, outside FP32 range, and the per-group exponent
    shift must bring each group's largest term back near 1.  Integrals are
    compared with the native FP64 kernel while they stay in normal FP64
    range."""
    import milkywayathome_client_gb300 as mw
    g = _setup(gpu_ctx, "three_streams")
    theta = np.asarray(g["theta"], dtype=np.float64).copy()
    theta[3] = mu      # stream 1: mu (degrees)
    theta[7] = sigma   # stream 1: sigma
    a = gpu_ctx.evaluate(theta, mw.MWSEP_PLAIN_F64)
    b = gpu_ctx.evaluate(theta, mw.MWSEP_PLAIN_DF)
    for x, y in zip(b.integrals, a.integrals):
        if abs(y) > 1e-280:
            assert _close_rel(x, y, REL), (x, y)
        else:
            assert abs(x) <= 1e-270, (x, y)
    if not (math.isnan(a.likelihood) or math.isinf(a.likelihood)):
        assert abs(a.likelihood - b.likelihood) <= ABS_LOGL, (a.likelihood, b.likelihood)


def test_double_float_star_table_respects_hbm_budget():
    """The per-star pair table is built on the first double-float
    evaluation; a context whose device-memory budget cannot hold it reports
    MWSEP_ERR_BUDGET, keeps working in the other forms, and builds it once
    the budget allows."""
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import native as N
    pf, sf, g = load_case("three_streams")
    sp = mw.StarPoints.read(sf)
    with mw.Context(0) as ctx:
        ctx.set_problem(mw.AstronomyParameters.read(pf))
        ctx.set_stars(sp)
        ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_F64)
        ctx.evaluate(g["theta"], mw.MWSEP_MIXED_F32)
        ctx.set_hbm_budget(ctx.device_bytes + 1024)
        with pytest.raises(mw.MwsepError) as e:
            ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_DF)
        assert e.value.status == N.MWSEP_ERR_BUDGET
        r = ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_F64)
        assert abs(r.likelihood - g["likelihood"]) <= ABS_LOGL
        before = ctx.device_bytes
        ctx.set_hbm_budget(0)
        r = ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_DF)
        assert abs(r.likelihood - g["likelihood"]) <= ABS_LOGL
        assert ctx.device_bytes - before >= 16 * sp.to_array().shape[0] * 20  # convolve 20


def test_double_float_first_use_from_threads():
    """Four contexts on four threads making their first double-float
    evaluation at once (a fresh process, so the exp2 table is not yet on
    the device): every result equals a single-threaded evaluation."""
    import subprocess
    import sys
    import textwrap
    pf, sf, g = load_case("three_streams")
    code = textwrap.dedent(f"""
        import threading, sys
        sys.path.insert(0, {repr(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))})
        import milkywayathome_client_gb300 as mw
        ap, sp = mw.AstronomyParameters.read({pf!r}), mw.StarPoints.read({sf!r})
        theta = {list(g["theta"])!r}
        ctxs = [mw.Context(0) for _ in range(4)]
        for c in ctxs:
            c.set_problem(ap); c.set_stars(sp)
        out = [None] * 4
        go = threading.Barrier(4)
        def run(i):
            go.wait()
            out[i] = ctxs[i].evaluate(theta, mw.MWSEP_PLAIN_DF)
        ths = [threading.Thread(target=run, args=(i,)) for i in range(4)]
        for t in ths: t.start()
        for t in ths: t.join()
        ref = ctxs[0].evaluate(theta, mw.MWSEP_PLAIN_DF)
        assert all(o.integrals == ref.integrals and o.likelihood == ref.likelihood for o in out)
        print("ok", ref.likelihood)
    """)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("ok")


def test_double_float_mixed_forms_batch(gpu_ctx):
    """General alpha/delta, alpha = delta = 1 and q = 0 thetas in one batch:
    each form's kernel skips the others' thetas, so every result equals its
    single evaluation bit for bit and stays within the plain bounds of the
    native FP64 kernel."""
    import milkywayathome_client_gb300 as mw
    g = _setup(gpu_ctx, "general_alpha_delta")
    base = np.asarray(g["theta"], dtype=np.float64)
    hern = base.copy()
    hern[0], hern[3] = 1.0, 1.0  # alpha, delta
    qzero = base.copy()
    qzero[1] = 0.0  # q
    thetas = [base, hern, base * (1 + 1e-3), hern * (1 - 1e-3), qzero]
    thetas[3][0], thetas[3][3] = 1.0, 1.0
    batch = gpu_ctx.evaluate_batch(thetas, mw.MWSEP_PLAIN_DF)
    for t, b in zip(thetas, batch):
        one = gpu_ctx.evaluate(t, mw.MWSEP_PLAIN_DF)
        assert one.integrals == b.integrals and one.likelihood == b.likelihood
        f64 = gpu_ctx.evaluate(t, mw.MWSEP_PLAIN_F64)
        for x, y in zip(b.integrals, f64.integrals):
            assert _close_rel(x, y, REL), (x, y)
        if math.isnan(f64.likelihood):
            assert math.isnan(b.likelihood)
        else:
            assert abs(b.likelihood - f64.likelihood) <= ABS_LOGL
