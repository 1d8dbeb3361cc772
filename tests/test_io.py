"""Host side of the drop-in: the reference's file formats, the theta layout,
the rank slicing and EVALUATION_STATE, through the C ABI (no GPU needed).
Fault injection on the host: malformed files and bad arguments return status
codes instead of exiting."""
import math
import os

import numpy as np
import pytest

import milkywayathome_client_gb300 as mw
from milkywayathome_client_gb300 import native as N
from conftest import CASES, GOLDEN, REFERENCE_DIR, golden_cases, load_case


@pytest.mark.parametrize("name", golden_cases())
def test_reads_golden_problem(built_library, oracle_built, name):
    pf, sf, g = load_case(name)
    ap = mw.AstronomyParameters.read(pf)
    o = oracle_built.Oracle(pf, sf)
    assert ap.optimized_parameter_count == len(g["theta"]) == o.n_theta
    assert ap.number_streams == o.n_streams
    assert ap.number_integrals == o.n_areas
    sp = mw.StarPoints.read(sf)
    assert sp.number_stars == o.n_stars


def test_write_read_round_trip(built_library, tmp_path):
    pf, sf, g = load_case("cut_area")
    ap = mw.AstronomyParameters.read(pf)
    out = tmp_path / "p.txt"
    ap.write(str(out))
    ap2 = mw.AstronomyParameters.read(str(out))
    assert ap2.optimized_parameter_count == ap.optimized_parameter_count
    assert ap2.number_integrals == 2
    for i in range(2):
        a, b = ap.area(i), ap2.area(i)
        for k in ("mu_steps", "nu_steps", "r_steps", "max_calculation"):
            assert a[k] == b[k]
        for k in ("mu_min", "mu_max", "nu_min", "r_max"):
            assert abs(a[k] - b[k]) < 1e-6
    # the reference writer prints stream weights with %lf (6 decimals), arrays with %.20lf
    np.testing.assert_allclose(ap2.search_parameters(), ap.search_parameters(), rtol=0, atol=5e-7)
    sp = mw.StarPoints.read(sf)
    sout = tmp_path / "s.txt"
    sp.write(str(sout))
    np.testing.assert_array_equal(mw.StarPoints.read(str(sout)).to_array(), sp.to_array())


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE_DIR, "tests")), reason="no reference fixtures")
@pytest.mark.parametrize("fname,count,areas", [("astronomy_parameters-86-small.txt", 8, 2),
                                               ("astronomy_parameters-11-small.txt", 20, 1),
                                               ("astronomy_parameters-79-small-aux.txt", 11, 1),
                                               ("astronomy_parameters-20-small.txt", 14, 1)])
def test_reads_reference_fixtures(built_library, fname, count, areas):
    ap = mw.AstronomyParameters.read(os.path.join(REFERENCE_DIR, "tests", fname))
    assert ap.optimized_parameter_count == count
    assert ap.number_integrals == areas


def _background(ap, n):
    return [ap.struct.background_parameters[i] for i in range(n)]


def test_aux_values_beyond_number_parameters(built_library, oracle_built, tmp_path):
    """The reference's astronomy_parameters-79-aux.txt lists seven background
    values under number_parameters 4: the search maps four of them (8
    parameters in all) and the aux profile reads values 4..6, as
    init_constants does; both writers keep the seven."""
    pf = os.path.join(GOLDEN, "reference_large", "79-aux", "params.txt")
    ap = mw.AstronomyParameters.read(pf)
    assert ap.struct.number_background_parameters == 4 and ap.struct.aux_bg_profile == 1
    assert ap.optimized_parameter_count == 8
    assert _background(ap, 7)[4:] == [100.0, 50.0, 25.0]
    assert oracle_built.Oracle(pf, os.path.join(CASES, "config0", "stars.txt")).n_theta == 8
    t = tmp_path / "p.txt"
    ap.write(str(t))
    back = mw.AstronomyParameters.read(str(t))
    assert back.struct.number_background_parameters == 4 and _background(back, 7) == _background(ap, 7)
    b = tmp_path / "p.mwsp"
    ap.write_binary(str(b))
    back = mw.AstronomyParameters.read_binary(str(b))
    assert back.struct.number_background_parameters == 4 and _background(back, 7) == _background(ap, 7)
    # an aux profile without its three values is refused
    lines = []
    for line in open(pf).read().splitlines():
        key, _, vals = line.partition(": ")
        if key.endswith("[7]") and not lines[-1].startswith("number_streams"):
            line = key.replace("[7]", "[4]") + ": " + ", ".join(vals.split(", ")[:4])
        lines.append(line)
    bad = tmp_path / "short.txt"
    bad.write_text("\n".join(lines) + "\n")
    with pytest.raises(mw.MwsepError):
        mw.AstronomyParameters.read(str(bad))


def test_theta_layout(built_library):
    """set_astronomy_parameters scatter order (cpu/parameters.c:332-363)."""
    pf, _, g = load_case("three_streams")
    ap = mw.AstronomyParameters.read(pf)
    t = np.arange(1, ap.optimized_parameter_count + 1, dtype=float)
    ap.set_parameters(t)
    np.testing.assert_array_equal(ap.search_parameters(), t)
    s = ap.struct
    assert s.background_parameters[1] == 1.0 and s.background_parameters[2] == 2.0
    assert s.stream_weights[0] == 3.0
    assert [s.stream_parameters[0][j] for j in range(5)] == [4.0, 5.0, 6.0, 7.0, 8.0]
    assert s.stream_weights[2] == 15.0
    with pytest.raises(ValueError):
        ap.set_parameters(t[:-1])


def test_split_matches_reference_formula(built_library):
    pf, sf, _ = load_case("ragged_sizes")
    for nranks in (1, 2, 3, 7):
        total = 0
        for r in range(nranks):
            ap = mw.AstronomyParameters.read(pf)
            ap.split(r, nranks)
            a = ap.area(0)
            cells = a["mu_steps"] * a["nu_steps"] * a["r_steps"]
            assert a["min_calculation"] == int(cells * (r / nranks))
            assert a["max_calculation"] == int(cells * ((r + 1) / nranks))
            total += a["max_calculation"] - a["min_calculation"]
        assert total == cells
    stars = mw.StarPoints.read(sf)
    n = stars.number_stars
    got = 0
    for r in range(4):
        sp = mw.StarPoints.read(sf)
        sp.split(r, 4)
        got += sp.number_stars
        assert sp.number_stars == int(n * ((r + 1) / 4)) - int(n * (r / 4))
    assert got == n


def test_initialize_state(built_library):
    pf, sf, _ = load_case("cut_area")
    ap = mw.AstronomyParameters.read(pf)
    sp = mw.StarPoints.read(sf)
    es = mw.EvaluationState(ap, sp)
    s = es.struct
    assert s.number_integrals == 2 and s.number_streams == 1 and s.total_stars == sp.number_stars
    ia = s.integral[1].contents
    assert ia.mu_steps == ap.area(1)["mu_steps"]
    assert abs(ia.mu_step_size - ap.area(1)["mu_step_size"]) < 1e-15
    assert ia.current_calculation == 0 and ia.max_calculation == ap.area(1)["max_calculation"]


@pytest.mark.parametrize("text", [
    "",                                                 # empty file
    "parameters_version: 0.04\nnumber_parameters: 4\n",  # truncated
    "parameters_version: 0.04\nnumber_parameters: 4\nbackground_weight: 0\n"
    "background_parameters[4]: 1, 0.7\n",                # short array
])
def test_malformed_parameter_file_returns_status(built_library, tmp_path, text):
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(mw.MwsepError) as e:
        mw.AstronomyParameters.read(str(p))
    assert e.value.status == N.MWSEP_ERR_IO


def test_missing_files_return_status(built_library, tmp_path):
    with pytest.raises(mw.MwsepError) as e:
        mw.AstronomyParameters.read(str(tmp_path / "nope.txt"))
    assert e.value.status == N.MWSEP_ERR_IO
    with pytest.raises(mw.MwsepError) as e:
        mw.StarPoints.read(str(tmp_path / "nope.txt"))
    assert e.value.status == N.MWSEP_ERR_IO
    bad = tmp_path / "stars.txt"
    bad.write_text("3\n1 2 3\n4 5\n")
    with pytest.raises(mw.MwsepError) as e:
        mw.StarPoints.read(str(bad))
    assert e.value.status == N.MWSEP_ERR_IO


def test_null_arguments_return_status(built_library):
    L = N.lib()
    assert L.mwsep_read_astronomy_parameters(None, None) == N.MWSEP_ERR_ARG
    assert L.mwsep_ctx_evaluate(None, None, 0, None) == N.MWSEP_ERR_ARG
    assert L.mwsep_last_error() == N.MWSEP_ERR_ARG
    v = L.mwsep_evaluate(None, None, None, None)
    assert math.isnan(v)


def test_status_strings(built_library):
    L = N.lib()
    for s in range(0, 11):
        assert L.mwsep_status_string(s)
    assert b"sm_103" in L.mwsep_version()
