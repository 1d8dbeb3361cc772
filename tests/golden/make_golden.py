"""Generate the golden fixtures under tests/golden/cases/.

Each case is a small synthetic wedge (parameter file + star file in the
reference's formats) plus the outputs of the REFERENCE's own CPU evaluator,
compiled from the reference sources by ``make -C oracle ref`` (oracle/_ref).
The reference sources are only needed when regenerating; the committed
fixtures travel with the repository.

Also records the reference's results on its own test fixtures
(tests/astronomy_parameters-*-small.txt with the theta vectors of
tests/CMakeLists.txt:24-41) as values only, in reference_fixtures.json,
the reference's stripe-frame transforms (stripe_normal /
sgr_stripe_normal + get_transform, transform_point; cpu/stCoords.c,
cpu/stVector.c) for a set of wedges and points, in transforms.json, and the
reference's matrix_invert (util/matrix.c) of seeded matrices, in
matrix_invert.json.

    python tests/golden/make_golden.py [--aux-only]
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from milkywayathome_client_gb300 import synthetic as syn  # noqa: E402
from oracle import oracle as orc  # noqa: E402

CASES = os.path.join(HERE, "cases")


def _wedge(mu, nu, r):
    return syn.Area(mu, nu, r)


def case_list():
    """(name, Problem, n_stars, seed) of every golden case."""
    cases = []
    rng = np.random.Generator(np.random.PCG64(20261203))

    def P(**kw):
        return syn.Problem(**kw)

    p = P(convolve=15, areas=[_wedge((310.0, 340.0, 20), (-1.25, 1.25, 10), (16.0, 22.5, 14))])
    p.streams = syn.draw_streams(rng, 1, 310.0, 340.0)
    cases.append(("basic_1stream", p, 600))

    p = P(convolve=20, areas=[_wedge((310.0, 420.0, 24), (-1.25, 1.25, 12), (16.0, 22.5, 16))])
    p.streams = syn.draw_streams(rng, 3, 310.0, 420.0)
    cases.append(("three_streams", p, 800))

    # a cut area subtracted from the wedge (as tests/astronomy_parameters-86)
    p = P(convolve=12, areas=[_wedge((310.0, 340.0, 16), (-1.25, 1.25, 8), (16.0, 22.5, 10)),
                              _wedge((320.0, 324.0, 6), (-1.25, 1.25, 5), (16.0, 22.5, 10))])
    p.streams = syn.draw_streams(rng, 1, 310.0, 340.0)
    cases.append(("cut_area", p, 500))

    # aux_bg_profile = 1 with a, b, c = 100, 50, 25 (the -aux fixtures)
    p = P(convolve=10, aux=(100.0, 50.0, 25.0),
          areas=[_wedge((310.0, 340.0, 12), (-1.25, 1.25, 6), (16.0, 22.5, 10))])
    p.streams = syn.draw_streams(rng, 2, 310.0, 340.0)
    cases.append(("aux_profile", p, 400))

    # general alpha/delta (pow branch, :259-272)
    p = P(convolve=10, alpha=1.3, delta=0.8, optimize_alpha_delta=True,
          areas=[_wedge((310.0, 340.0, 12), (-1.25, 1.25, 6), (16.0, 22.5, 10))])
    p.streams = syn.draw_streams(rng, 1, 310.0, 340.0)
    cases.append(("general_alpha_delta", p, 400))

    # Sagittarius coordinates (gcToSgr / sgrToGal)
    p = P(convolve=10, sgr=1, wedge=79,
          areas=[_wedge((135.0, 235.0, 14), (-1.25, 1.25, 6), (16.0, 22.5, 10))])
    p.streams = syn.draw_streams(rng, 2, 135.0, 235.0)
    cases.append(("sgr_coordinates", p, 400))

    # a stream switched off by |sigma| < 1e-4 (:279-280) beside a live one
    p = P(convolve=10, areas=[_wedge((310.0, 340.0, 12), (-1.25, 1.25, 6), (16.0, 22.5, 10))])
    p.streams = syn.draw_streams(rng, 2, 310.0, 340.0)
    p.streams[1].sigma = 0.00005
    cases.append(("stream_off", p, 400))

    # four streams (the reference CUDA path's maximum) with convolve 120
    p = P(convolve=120, areas=[_wedge((310.0, 340.0, 8), (-1.25, 1.25, 4), (16.0, 22.5, 6))])
    p.streams = syn.draw_streams(rng, 4, 310.0, 340.0)
    cases.append(("four_streams_c120", p, 300))

    # more streams than the reference CUDA path allowed
    p = P(convolve=8, areas=[_wedge((310.0, 340.0, 10), (-1.25, 1.25, 5), (16.0, 22.5, 8))])
    p.streams = syn.draw_streams(rng, 6, 310.0, 340.0)
    cases.append(("six_streams", p, 300))

    # ragged / minimal sizes: one cell, one convolution point, one star
    p = P(convolve=1, areas=[_wedge((320.0, 321.0, 1), (-0.5, 0.5, 1), (18.0, 19.0, 1))])
    p.streams = syn.draw_streams(rng, 1, 320.0, 321.0)
    cases.append(("single_cell_single_star", p, 1))

    # odd sizes that are not multiples of any block or warp
    p = P(convolve=7, areas=[_wedge((310.0, 340.0, 13), (-1.25, 1.25, 7), (16.0, 22.5, 11))])
    p.streams = syn.draw_streams(rng, 2, 310.0, 340.0)
    cases.append(("ragged_sizes", p, 333))

    # the shape of config 0 at full size (80 x 40 x 70, convolve 30), 10k stars
    c0 = syn.config(0)
    cases.append(("config0", c0["problems"][0], 10_000))

    # the library's maximum sizes: 8 streams, 8 integral areas (a wedge and
    # 7 cuts), convolve 512, on a small grid
    p = P(convolve=512, areas=[_wedge((310.0, 340.0, 8), (-1.25, 1.25, 4), (16.0, 22.5, 6))] +
          [_wedge((311.0 + 3.5 * i, 313.0 + 3.5 * i, 2), (-1.25, 1.25, 2), (16.0, 22.5, 6)) for i in range(7)])
    p.streams = syn.draw_streams(rng, 8, 310.0, 340.0)
    cases.append(("max_limits", p, 64))
    return cases


def reference_on_fixtures(ref_dir):
    """The reference's own results on its own small test fixtures."""
    t = os.path.join(ref_dir, "tests")
    p1 = [0.571713, 12.312119, -3.305187, 148.010257, 22.453902, 0.42035, -0.468858, 0.760579, -1.361644,
          177.884238, 23.882892, 1.210639, -1.611974, 8.534378, -1.361644, 177.884238, 10.882892, 1.210639,
          -1.611974, 8.534378]
    p79 = [0.34217373320392042, 25.9517910846623, -2.1709414738826602, 38.272511356953906, 30.225190442596112,
           2.2149060013372885, 0.32316169064291655, 2.7740244716285285]
    p86 = [0.73317163557524425, 14.657212876628332, -1.7054653473950408, 16.911711745343633,
           28.077212666463502, -1.2032908515814611, 3.5273606439247287, 2.2248214505875008]
    out = {}
    for n, theta, S, A in [(79, p79, 1, 1), (86, p86, 1, 2), (11, p1, 3, 1), (12, p1, 3, 1)]:
        pf = os.path.join(t, f"astronomy_parameters-{n}-small.txt")
        sf = os.path.join(t, f"stars-{n}.txt")
        r = orc.Reference.evaluate(pf, sf, theta, S, A)
        r.pop("seconds")
        r["theta"] = theta
        r["params_file"] = f"tests/astronomy_parameters-{n}-small.txt"
        r["stars_file"] = f"tests/stars-{n}.txt"
        out[str(n)] = r
    return out


def reference_transforms():
    """The reference's stripe rotation for survey and Sgr wedges, and
    transform_point of seeded Galactic points through each."""
    rng = np.random.Generator(np.random.PCG64(4242))
    out = []
    for sgr, wedges in ((0, [9, 10, 11, 12, 20, 37, 46, 47, 60, 79, 82, 86]), (1, [5, 20, 79, 100, 130])):
        for w in wedges:
            m = orc.Reference.stripe_transform(sgr, w)
            pts = []
            for _ in range(4):
                l, b, r = rng.uniform(0, 360), rng.uniform(-80, 80), rng.uniform(16, 23)
                xyz = orc.Oracle.lbr_to_xyz(l, b, r)
                pts.append({"lbr": [l, b, r], "xyz": [float(v) for v in xyz],
                            "out": [float(v) for v in orc.Reference.transform_point(xyz, m)]})
            out.append({"sgr": sgr, "wedge": w, "matrix": [float(v) for v in m.ravel()], "points": pts})
    return out


def reference_inversions():
    """matrix_invert of seeded well-conditioned matrices (Hessian-like:
    symmetric negative definite, sizes 1..23) and of a general one."""
    rng = np.random.Generator(np.random.PCG64(777))
    out = []
    for n in (1, 2, 3, 5, 8, 13, 23):
        a = rng.standard_normal((n, n))
        h = -(a @ a.T + n * np.eye(n)) * 10.0 ** rng.uniform(-2, 4)
        out.append({"a": h.ravel().tolist(), "n": n, "inverse": orc.Reference.invert_matrix(h).ravel().tolist()})
    g = rng.standard_normal((6, 6))
    out.append({"a": g.ravel().tolist(), "n": 6, "inverse": orc.Reference.invert_matrix(g).ravel().tolist()})
    return out


def main():
    orc.build(reference=True)
    if not orc.reference_available():
        sys.exit("the reference sources are needed to regenerate the goldens")
    with open(os.path.join(HERE, "transforms.json"), "w") as f:
        json.dump(reference_transforms(), f, indent=1)
    with open(os.path.join(HERE, "matrix_invert.json"), "w") as f:
        json.dump(reference_inversions(), f, indent=1)
    if "--aux-only" in sys.argv:
        return
    os.makedirs(CASES, exist_ok=True)
    index = {}
    for k, (name, p, n) in enumerate(case_list()):
        d = os.path.join(CASES, name)
        os.makedirs(d, exist_ok=True)
        pf = os.path.join(d, "params.txt")
        sf = os.path.join(d, "stars.txt")
        p.write(pf)
        stars = syn.sample_stars(p, n, np.random.Generator(np.random.PCG64(7000 + k)))
        syn.write_stars(sf, stars)
        theta = [float(x) for x in p.theta()]
        r = orc.Reference.evaluate(pf, sf, theta, len(p.streams), len(p.areas))
        r.pop("seconds")
        r["theta"] = theta
        with open(os.path.join(d, "golden.json"), "w") as f:
            json.dump(r, f, indent=1)
        index[name] = {"streams": len(p.streams), "areas": len(p.areas), "convolve": p.convolve,
                       "stars": n, "cells": p.cells()}
        print(name, r["likelihood"])
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1)
    ref = orc.REF_SRC
    if os.path.isdir(os.path.join(ref, "tests")):
        with open(os.path.join(HERE, "reference_fixtures.json"), "w") as f:
            json.dump(reference_on_fixtures(ref), f, indent=1)


if __name__ == "__main__":
    main()
