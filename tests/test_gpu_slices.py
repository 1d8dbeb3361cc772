"""Cell-range slices on the GPU against the reference's own sliced evaluations.

A rank's share of an evaluation (split_astronomy_parameters and
split_star_points, cpu/parameters.c:502-522, cpu/star_points.c:105-131)
integrates only the cells [min_calculation, max_calculation) of each area
(cpu/evaluation_optimized.c:521-527) and evaluates its own stars against
those partial integrals.  Goldens: the reference's CPU evaluator run with the
same split (tests/golden/make_scale_golden.py): 3 ranks of config0 and
cut_area (two areas), 8 ranks of the full-size config 1.

Every path that integrates takes the slice: the context API in the three
forms, batches, the EvalFunc entries (which read the range from
EVALUATION_STATE, as calculate_integral does) and the tiled engine.  The
ranks' cut-subtracted integrals composed as the reference's integral_compose
does (cpu/astronomy_worker.c:67-92) equal the whole evaluation.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import CASES, load_case

pytestmark = pytest.mark.gpu

REL_INT = 1e-12
ABS_LOGL = 1e-12
MIXED_REL_INT = 1e-6
ABS_LOGL_MIXED = 1e-7


def _rel(a, b):
    if b == 0.0:
        return 0.0 if a == 0.0 else math.inf
    return abs(a - b) / abs(b)


def _slices(name):
    with open(os.path.join(CASES, name, "golden_slices.json")) as f:
        return json.load(f)


def _split_inputs(pf, sf, rank, nranks):
    import milkywayathome_client_gb300 as mw
    ap = mw.AstronomyParameters.read(pf)
    sp = mw.StarPoints.read(sf)
    ap.split(rank, nranks)
    sp.split(rank, nranks)
    return ap, sp


def _check(areas, likelihood, g, rel, dl, label):
    for a, (got, want) in enumerate(zip(areas, g["area_integrals"])):
        for k, (x, y) in enumerate(zip(got, want)):
            assert _rel(x, y) <= rel, f"{label}: area {a} component {k}: {x!r} vs {y!r}"
    if likelihood is not None:
        assert abs(likelihood - g["likelihood"]) <= dl, f"{label}: logL {likelihood!r} vs {g['likelihood']!r}"


@pytest.mark.parametrize("name", ["config0", "cut_area"])
def test_context_slices_all_forms(gpu_ctx, name):
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import sharding
    pf, sf, whole = load_case(name)
    gs = _slices(name)
    per_form = {}
    for g in gs:
        ap, sp = _split_inputs(pf, sf, g["rank"], g["nranks"])
        gpu_ctx.set_problem(ap)
        gpu_ctx.set_stars(sp)
        for prec, rel, dl in ((mw.MWSEP_PLAIN_F64, REL_INT, ABS_LOGL), (mw.MWSEP_PLAIN_DF, REL_INT, ABS_LOGL),
                              (mw.MWSEP_MIXED_F32, MIXED_REL_INT, ABS_LOGL_MIXED)):
            r = gpu_ctx.evaluate(g["theta"], prec)
            _check(r.area_integrals, r.likelihood, g, rel, dl, f"{name} rank {g['rank']} form {prec}")
            per_form.setdefault(prec, []).append(r.integrals)
            # a batch takes the slice too
            b = gpu_ctx.evaluate_batch([g["theta"], g["theta"]], prec)
            assert b[0].integrals == r.integrals and b[1].integrals == r.integrals
    want = [whole["background_integral"]] + whole["stream_integrals"]
    for prec, rows in per_form.items():
        tol = REL_INT if prec != mw.MWSEP_MIXED_F32 else MIXED_REL_INT
        for x, y in zip(sharding.integral_compose(rows), want):
            assert _rel(x, y) <= tol, (prec, x, y)
    # the whole problem again on the same resident tables: every cell
    ap = mw.AstronomyParameters.read(pf)
    gpu_ctx.set_problem(ap)
    gpu_ctx.set_stars(mw.StarPoints.read(sf))
    r = gpu_ctx.evaluate(whole["theta"], mw.MWSEP_PLAIN_F64)
    _check(r.area_integrals, r.likelihood, whole, REL_INT, ABS_LOGL, f"{name} whole after slices")


@pytest.mark.parametrize("name", ["config0", "cut_area"])
def test_evalfunc_slices(built_library, name):
    """The EvalFunc entries integrate the state's [min_calculation,
    max_calculation) of each area, as cpu_evaluate does."""
    import milkywayathome_client_gb300 as mw
    pf, sf, _ = load_case(name)
    for g in _slices(name):
        ap, sp = _split_inputs(pf, sf, g["rank"], g["nranks"])
        for fn, rel, dl in ((mw.evaluate, REL_INT, ABS_LOGL), (mw.evaluate_df, REL_INT, ABS_LOGL),
                            (mw.evaluate_mixed, MIXED_REL_INT, ABS_LOGL_MIXED)):
            es = mw.EvaluationState(ap, sp)
            v = fn(g["theta"], ap, es, sp)
            _check(es.area_integrals, v - 3.0, g, rel, dl, f"{name} rank {g['rank']} {fn.__name__}")
            for a in range(ap.number_integrals):
                ia = es.struct.integral[a].contents
                assert ia.current_calculation == ia.max_calculation  # where the walk stopped


@pytest.mark.parametrize("name", ["config0", "cut_area"])
def test_engine_slices(built_library, name):
    """Split wedges resident side by side in the tiled engine, one request
    per rank in one batch."""
    import milkywayathome_client_gb300 as mw
    pf, sf, _ = load_case(name)
    gs = _slices(name)
    with mw.Context(0) as ctx:
        wids = [ctx.add_wedge(*_split_inputs(pf, sf, g["rank"], g["nranks"])) for g in gs]
        for prec, rel, dl in ((mw.MWSEP_PLAIN_F64, REL_INT, ABS_LOGL), (mw.MWSEP_MIXED_F32, MIXED_REL_INT,
                                                                        ABS_LOGL_MIXED),
                              (mw.MWSEP_PLAIN_DF, REL_INT, ABS_LOGL)):
            res = ctx.evaluate_requests([(w, g["theta"]) for w, g in zip(wids, gs)], prec)
            for r, g in zip(res, gs):
                _check(r.area_integrals, r.likelihood, g, rel, dl, f"engine {name} rank {g['rank']} form {prec}")


def test_config1_slices(gpu_ctx, golden_inputs):
    """The full-size wedge (1600 x 640 x 140 cells, convolve 120) in 8 rank
    slices, each against the reference's own slice."""
    import milkywayathome_client_gb300 as mw
    pf, sf, G = golden_inputs("scale", "config1")
    for g in G["slices"]:
        ap, sp = _split_inputs(pf, sf, g["rank"], g["nranks"])
        gpu_ctx.set_problem(ap)
        gpu_ctx.set_stars(sp)
        for prec, rel, dl in ((mw.MWSEP_PLAIN_DF, REL_INT, ABS_LOGL), (mw.MWSEP_MIXED_F32, MIXED_REL_INT,
                                                                        ABS_LOGL_MIXED)):
            r = gpu_ctx.evaluate(g["theta"], prec)
            _check(r.area_integrals, r.likelihood, g, rel, dl, f"config1 rank {g['rank']} form {prec}")
    # the plain FP64 form on two ranks (2 s per whole evaluation)
    for g in (G["slices"][0], G["slices"][5]):
        ap, sp = _split_inputs(pf, sf, g["rank"], g["nranks"])
        gpu_ctx.set_problem(ap)
        gpu_ctx.set_stars(sp)
        r = gpu_ctx.evaluate(g["theta"], mw.MWSEP_PLAIN_F64)
        _check(r.area_integrals, r.likelihood, g, REL_INT, ABS_LOGL, f"config1 rank {g['rank']} plain")


def test_negative_slice_start_refused(gpu_ctx):
    """A negative min_calculation lies outside the reference's domain (its
    get_steps would index before the grid): refused with MWSEP_ERR_ARG."""
    import milkywayathome_client_gb300 as mw
    pf, _, _ = load_case("basic_1stream")
    ap = mw.AstronomyParameters.read(pf)
    ap.struct.integral[0].contents.min_calculation = -1
    with pytest.raises(mw.MwsepError):
        gpu_ctx.set_problem(ap)


@pytest.mark.parametrize("name", ["aux_profile", "general_alpha_delta", "sgr_coordinates", "six_streams"])
def test_slices_other_forms_against_oracle(gpu_ctx, oracle_built, name):
    """Rank slices of the background forms and coordinate frames the two
    reference-sliced cases do not cover (the aux profile and general
    alpha/delta, whose column-independent shares the double-float form sums
    box by box; Sagittarius coordinates; eight-stream kernels), against the
    oracle's sliced integrals (the oracle equals the reference's own sliced
    runs on config0 and cut_area); and q = 0, whose background the
    double-float form also sums box by box."""
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case(name)
    o = oracle_built.Oracle(pf, sf)
    theta_q0 = list(g["theta"])
    ap0 = mw.AstronomyParameters.read(pf)
    q_index = 1 if ap0.struct.background_optimize[0] else 0  # q follows alpha when alpha is optimised
    theta_q0[q_index] = 0.0
    for rank in range(3):
        ap, sp = _split_inputs(pf, sf, rank, 3)
        gpu_ctx.set_problem(ap)
        gpu_ctx.set_stars(sp)
        _, want = o.integrals(g["theta"], rank=rank, nranks=3)
        for prec, rel in ((mw.MWSEP_PLAIN_F64, REL_INT), (mw.MWSEP_PLAIN_DF, REL_INT), (mw.MWSEP_MIXED_F32, 2e-6)):
            r = gpu_ctx.evaluate(g["theta"], prec)
            _check(r.area_integrals, None, {"area_integrals": want.tolist()}, rel, None,
                   f"{name} rank {rank} form {prec}")
        _, want0 = o.integrals(theta_q0, rank=rank, nranks=3)
        for prec in (mw.MWSEP_PLAIN_F64, mw.MWSEP_PLAIN_DF):
            r = gpu_ctx.evaluate(theta_q0, prec)
            assert _rel(r.area_integrals[0][0], want0[0][0]) <= REL_INT, (name, rank, prec)
