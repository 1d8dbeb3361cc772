"""Optimiser-side host pieces on the CPU: the matrix inversion and the
errors() arithmetic against the reference's own util/matrix.c
(tests/golden/matrix_invert.json, made by the compiled reference; live where
it is compiled), the step/bounds getters against the parameter file, and
the errors file format."""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_case


def _inversions():
    with open(os.path.join(GOLDEN, "matrix_invert.json")) as f:
        return json.load(f)


def test_invert_matrix_matches_reference_fixture(built_library):
    import milkywayathome_client_gb300 as mw
    for case in _inversions():
        n = case["n"]
        a = np.array(case["a"]).reshape(n, n)
        got = mw.invert_matrix(a)
        assert got.ravel().tolist() == case["inverse"], n


def test_invert_matrix_matches_live_reference(built_library, oracle_built):
    import milkywayathome_client_gb300 as mw
    orc = oracle_built
    if not orc.reference_available():
        pytest.skip("reference not compiled here")
    rng = np.random.default_rng(3)
    for n in (4, 7, 11, 17):
        a = rng.standard_normal((n, n)) * 10.0 ** rng.uniform(-3, 3, size=(n, n))
        assert np.array_equal(mw.invert_matrix(a), orc.Reference.invert_matrix(a)), n


def test_invert_matrix_singular_is_an_error(built_library):
    import milkywayathome_client_gb300 as mw
    with pytest.raises(mw.MwsepError):
        mw.invert_matrix(np.zeros((3, 3)))
    with pytest.raises(mw.MwsepError):
        mw.invert_matrix(np.array([[1.0, 2.0], [2.0, 4.0]]) * 0.0)


def test_errors_from_hessian(built_library):
    import milkywayathome_client_gb300 as mw
    rng = np.random.default_rng(8)
    a = rng.standard_normal((5, 5))
    H = -(a @ a.T + 5 * np.eye(5))
    sigma, sd = mw.errors_from_hessian(H, 1000)
    inv = mw.invert_matrix(H)
    assert np.array_equal(sigma, inv / 1000.0)
    assert sd.tolist() == [math.sqrt(abs(sigma[i, i])) for i in range(5)]
    np.testing.assert_allclose(sigma, np.linalg.inv(H) / 1000, rtol=1e-12)


def test_write_errors_format(built_library, tmp_path):
    import milkywayathome_client_gb300 as mw
    H = np.array([[-2.0, 0.5], [0.5, -1.0]])
    sigma, sd = mw.errors_from_hessian(H, 4)
    p = str(tmp_path / "errors.txt")
    mw.write_errors(p, H, sigma, sd)
    lines = open(p).read().splitlines()
    assert lines[0] == "hessian [2 x 2]:"
    assert lines[1] == " -2.00000000000000000000 0.50000000000000000000"
    assert lines[3] == "" and lines[4] == "SIGMA:"
    assert lines[7] == "" and lines[8].startswith("Errors:")
    assert [float(x) for x in lines[9].split()] == pytest.approx(sd.tolist(), abs=1e-6)


def test_step_and_bounds_follow_theta_layout(built_library):
    import milkywayathome_client_gb300 as mw
    pf, _, g = load_case("three_streams")
    ap = mw.AstronomyParameters.read(pf)
    st = ap.step()
    lo, hi = ap.bounds()
    P = ap.optimized_parameter_count
    assert st.shape == lo.shape == hi.shape == (P,)
    s = ap.struct
    want_step, want_lo, want_hi = [], [], []
    for i in range(s.number_background_parameters):
        if s.background_optimize[i]:
            want_step.append(s.background_step[i])
            want_lo.append(s.background_min[i])
            want_hi.append(s.background_max[i])
    for i in range(s.number_streams):
        if s.stream_weight_optimize[i]:
            want_step.append(s.stream_weight_step[i])
            want_lo.append(s.stream_weight_min[i])
            want_hi.append(s.stream_weight_max[i])
        for j in range(s.number_stream_parameters):
            if s.stream_optimize[i][j]:
                want_step.append(s.stream_step[i][j])
                want_lo.append(s.stream_min[i][j])
                want_hi.append(s.stream_max[i][j])
    assert st.tolist() == want_step and lo.tolist() == want_lo and hi.tolist() == want_hi
