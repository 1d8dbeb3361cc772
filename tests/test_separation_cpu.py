"""Separation output on the CPU: the oracle's restatement of
cpu/separation.c against the reference's own stripe transforms
(tests/golden/transforms.json, made by the reference's compiled
stCoords.c / stVector.c) and against its own per-star densities; the
library's host-side stripe rotation against the same fixture."""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, load_case


def _transforms():
    with open(os.path.join(GOLDEN, "transforms.json")) as f:
        return json.load(f)


def test_oracle_stripe_transform_matches_reference_fixture(oracle_built):
    orc = oracle_built
    for t in _transforms():
        m = orc.Oracle.stripe_transform(t["sgr"], t["wedge"])
        assert m.ravel().tolist() == t["matrix"], (t["sgr"], t["wedge"])


def test_oracle_transform_point_matches_reference_fixture(oracle_built):
    orc = oracle_built
    for t in _transforms():
        m = np.array(t["matrix"]).reshape(3, 3)
        for p in t["points"]:
            xyz = orc.Oracle.lbr_to_xyz(*p["lbr"])
            assert xyz.tolist() == p["xyz"]
            assert orc.Oracle.transform_point(xyz, m).tolist() == p["out"], (t["wedge"], p["lbr"])


def test_oracle_transforms_match_live_reference(oracle_built):
    orc = oracle_built
    if not orc.reference_available():
        pytest.skip("reference not compiled here")
    rng = np.random.default_rng(5)
    for sgr in (0, 1):
        for w in rng.integers(1, 140, size=12):
            a = orc.Oracle.stripe_transform(sgr, int(w))
            b = orc.Reference.stripe_transform(sgr, int(w))
            assert np.array_equal(a, b), (sgr, w)
            for _ in range(3):
                xyz = orc.Oracle.lbr_to_xyz(rng.uniform(0, 360), rng.uniform(-85, 85), rng.uniform(15, 24))
                assert np.array_equal(orc.Oracle.transform_point(xyz, a), orc.Reference.transform_point(xyz, b))


def test_library_stripe_transform_matches_reference_fixture(built_library):
    import milkywayathome_client_gb300 as mw
    for t in _transforms():
        m = mw.stripe_transform(t["sgr"], t["wedge"])
        assert m.ravel().tolist() == t["matrix"], (t["sgr"], t["wedge"])


def test_library_stripe_transform_rejects_bad_frame(built_library):
    import milkywayathome_client_gb300 as mw
    with pytest.raises(mw.MwsepError):
        mw.stripe_transform(2, 10)


def _weights(pf, theta):
    import milkywayathome_client_gb300 as mw
    ap = mw.AstronomyParameters.read(pf)
    ap.set_parameters(theta)
    return np.array([ap.struct.stream_weights[j] for j in range(ap.number_streams)])


@pytest.mark.parametrize("name", ["basic_1stream", "three_streams", "six_streams", "sgr_coordinates",
                                  "aux_profile", "cut_area"])
def test_oracle_separation_from_densities(oracle_built, built_library, name):
    """sprob and expected restated from the oracle's per-star densities
    (the quantities the likelihood goldens pin) with separation.c's
    weights: epsilon_s = e^w_s / (1 + sum e^w), epsilon_b = 1 / (1 + sum e^w)."""
    orc = oracle_built
    pf, sf, g = load_case(name)
    o = orc.Oracle(pf, sf)
    theta = g["theta"]
    ints, _ = o.integrals(theta)
    sprob, xyz, expected = o.separation(theta, ints)
    bg, st = o.star_densities(theta)
    w = _weights(pf, theta)
    denom = 1.0
    for x in w:
        denom += math.exp(x)
    eps = np.array([math.exp(x) / denom for x in w])
    pbx = (1.0 / denom) * bg / ints[0]
    psg = eps[None, :] * st / np.asarray(ints[1:])[None, :]
    want = psg / (psg.sum(axis=1, keepdims=True) + pbx[:, None])
    np.testing.assert_allclose(sprob, want, rtol=1e-14, atol=0)
    assert np.all(sprob >= 0) and np.all(sprob.sum(axis=1) <= 1 + 1e-15)
    np.testing.assert_allclose(expected, sprob.sum(axis=0), rtol=1e-12)
    assert xyz.shape == (o.n_stars, 3) and np.all(np.isfinite(xyz))


def test_oracle_separation_matches_golden_integrals(oracle_built):
    """With the reference's own integrals, the oracle's sprob is a
    probability vector for every star of every case with live streams."""
    orc = oracle_built
    for name in golden_cases():
        if name == "stream_off":
            continue
        pf, sf, g = load_case(name)
        o = orc.Oracle(pf, sf)
        ints = [g["background_integral"]] + list(g["stream_integrals"])
        sprob, _, expected = o.separation(g["theta"], ints)
        s = sprob.sum(axis=1)
        assert np.all((s >= 0) & (s <= 1 + 1e-15)), name
        assert 0 <= sum(expected) <= o.n_stars + 1e-9, name


def test_write_separation_file_format(built_library, tmp_path):
    import milkywayathome_client_gb300 as mw
    a = np.array([0, 2, 1], dtype=np.int32)
    x = np.array([[1.5, -2.25, 3.0], [0.0, 1e-7, -4.125], [10.0, 20.0, 30.0]])
    p = str(tmp_path / "sep.txt")
    mw.write_separation(p, a, x)
    lines = open(p).read().splitlines()
    assert lines == ["0 1.500000 -2.250000 3.000000", "2 0.000000 0.000000 -4.125000",
                     "1 10.000000 20.000000 30.000000"]
    with pytest.raises(ValueError):
        mw.write_separation(p, a, x[:2])
