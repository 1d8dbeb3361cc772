"""Golden fixtures at the reference's own inputs and at the benchmark sizes.

Every number here is written by the REFERENCE's own CPU evaluator, compiled
from the reference sources by ``make -C oracle ref`` (oracle/_ref).  The
reference sources are only needed when regenerating; what this script
writes travels with the repository:

  --fixtures   tests/golden/reference/<id>/: the reference's test fixtures
               tests/astronomy_parameters-<n>-small[-aux].txt and
               tests/stars-<n>.txt (the star file xz-compressed, byte for byte
               the reference's text) with the theta vectors of
               tests/CMakeLists.txt:24-41, and golden.json (per-area and final
               integrals, prob_sum, num_zero, likelihood).  Fixtures whose
               theta in tests/CMakeLists.txt has the wrong length are given
               the corrected vector described in CORRECTED below.
  --config K   tests/golden/scale/config<K>/ for benchmark config 1 or 2:
               params.txt, stars.txt.xz and golden.json with the reference's
               full single-core evaluation of each theta and, for config 1,
               its rank slices (split_astronomy_parameters /
               split_star_points, cpu/parameters.c:502-522,
               cpu/star_points.c:105-131) over 8 ranks.
  --slices     golden_slices.json beside the small synthetic cases config0
               and cut_area: every rank of a 3-way split.
  --large ID   tests/golden/reference_large/<ID>/ for the reference's large
               fixture tests/astronomy_parameters-<ID>.txt (ID 86, 12, 79 and
               the -aux files of 79, 86, 11, 12, with the theta of the small
               ones -- but 79-aux, whose number_parameters 4 leaves its aux
               values out of the search, takes test 79's; 1600 x 640 x 1400
               cells, ~1.7e11 points; the star file is the small fixture's):
               the reference's distributed evaluation over 8 ranks -- each
               rank's slice integrated by the reference, the slices summed in
               rank order as integral_compose does (cpu/astronomy_worker.c:
               67-92), then the reference's calculate_likelihood over the whole
               catalogue against that sum (likelihood_f, :94-121).

    python tests/golden/make_scale_golden.py --fixtures --slices --config 2 --config 1
"""
from __future__ import annotations

import json
import lzma
import multiprocessing as mp
import os
import shutil
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from milkywayathome_client_gb300 import synthetic as syn  # noqa: E402
from oracle import oracle as orc  # noqa: E402

REF_TESTS = os.path.join(orc.REF_SRC, "tests")
FIXDIR = os.path.join(HERE, "reference")
SCALEDIR = os.path.join(HERE, "scale")

# theta vectors of tests/CMakeLists.txt:24-41
PARAM_SET1 = [0.571713, 12.312119, -3.305187, 148.010257, 22.453902, 0.42035, -0.468858, 0.760579, -1.361644,
              177.884238, 23.882892, 1.210639, -1.611974, 8.534378, -1.361644, 177.884238, 10.882892, 1.210639,
              -1.611974, 8.534378]
TEST_79 = [0.34217373320392042, 25.9517910846623, -2.1709414738826602, 38.272511356953906, 30.225190442596112,
           2.2149060013372885, 0.32316169064291655, 2.7740244716285285]
TEST_86 = [0.73317163557524425, 14.657212876628332, -1.7054653473950408, 16.911711745343633,
           28.077212666463502, -1.2032908515814611, 3.5273606439247287, 2.2248214505875008]
AUX_ABC = [100.0, 50.0, 25.0]  # the -aux parameter files' background_parameters[4..6]

# CORRECTED: tests/CMakeLists.txt gives tests 20 and 21 (two streams, 14
# optimised parameters) the 20-value param_set1; they take its first 14
# values (q, r0 and the first two streams).  The -aux files optimise a, b, c
# too (2 + 3 + 6S values); they take the test's vector with the files' own
# a, b, c inserted after q and r0.
FIXTURES = [
    ("79", "79-small", "79", TEST_79),
    ("86", "86-small", "86", TEST_86),
    ("11", "11-small", "11", PARAM_SET1),
    ("12", "12-small", "12", PARAM_SET1),
    ("20", "20-small", "20", PARAM_SET1[:14]),
    ("21", "21-small", "21", PARAM_SET1[:14]),
    ("79-aux", "79-small-aux", "79", TEST_79[:2] + AUX_ABC + TEST_79[2:]),
    ("86-aux", "86-small-aux", "86", TEST_86[:2] + AUX_ABC + TEST_86[2:]),
    ("11-aux", "11-small-aux", "11", PARAM_SET1[:2] + AUX_ABC + PARAM_SET1[2:]),
    ("12-aux", "12-small-aux", "12", PARAM_SET1[:2] + AUX_ABC + PARAM_SET1[2:]),
]


def _dims(param_path):
    """(number of streams, number of integral areas) of a parameter file."""
    S = A = None
    with open(param_path) as f:
        for line in f:
            if line.startswith("number_streams:"):
                S = int(line.split(":")[1].split(",")[0])
            if line.startswith("number_cuts:"):
                A = 1 + int(line.split(":")[1])
    return S, A


def _ref_job(job):
    pf, sf, theta, rank, nranks = job
    S, A = _dims(pf)
    t0 = time.time()
    r = orc.Reference.evaluate(pf, sf, theta, S, A, rank=rank, nranks=nranks)
    r.pop("seconds")
    r["theta"] = [float(x) for x in theta]
    r["rank"], r["nranks"] = rank, nranks
    r["wall_s"] = round(time.time() - t0, 2)
    return r


def _run(jobs, procs=None):
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs or os.cpu_count()) as pool:
        return pool.map(_ref_job, jobs, chunksize=1)


def _xz(src, dst):
    with open(src, "rb") as f:
        data = f.read()
    with lzma.open(dst, "wb", preset=9 | lzma.PRESET_EXTREME) as f:
        f.write(data)


def unpack_stars(xz_path, out_path):
    """The star file as the reference read it (decompressed)."""
    with lzma.open(xz_path, "rb") as f, open(out_path, "wb") as g:
        shutil.copyfileobj(f, g)
    return out_path


def make_fixtures():
    os.makedirs(FIXDIR, exist_ok=True)
    jobs, dirs = [], []
    for fid, pname, sname, theta in FIXTURES:
        d = os.path.join(FIXDIR, fid)
        os.makedirs(d, exist_ok=True)
        shutil.copyfile(os.path.join(REF_TESTS, f"astronomy_parameters-{pname}.txt"), os.path.join(d, "params.txt"))
        jobs.append((os.path.join(d, "params.txt"), os.path.join(REF_TESTS, f"stars-{sname}.txt"), theta, 0, 1))
        dirs.append((d, fid, pname, sname))
    stars_done = {}
    for d, fid, pname, sname in dirs:
        # one compressed copy per star file, kept beside its first fixture
        if sname not in stars_done:
            _xz(os.path.join(REF_TESTS, f"stars-{sname}.txt"), os.path.join(d, "stars.txt.xz"))
            stars_done[sname] = fid
    results = _run(jobs)
    index = {}
    for (d, fid, pname, sname), r in zip(dirs, results):
        r["params_file"] = f"tests/astronomy_parameters-{pname}.txt"
        r["stars_file"] = f"tests/stars-{sname}.txt"
        r["stars_xz"] = os.path.relpath(os.path.join(FIXDIR, stars_done[sname], "stars.txt.xz"), HERE)
        with open(os.path.join(d, "golden.json"), "w") as f:
            json.dump(r, f, indent=1)
        index[fid] = {"params": os.path.relpath(os.path.join(d, "params.txt"), HERE), "stars_xz": r["stars_xz"]}
        print(fid, r["likelihood"], r["wall_s"], "s", flush=True)
    with open(os.path.join(FIXDIR, "index.json"), "w") as f:
        json.dump(index, f, indent=1)


def make_config(k, work):
    d = os.path.join(SCALEDIR, f"config{k}")
    os.makedirs(d, exist_ok=True)
    m = syn.materialise(k, os.path.join(work, f"config{k}"))
    fi = m["files"][0]
    shutil.copyfile(fi["params"], os.path.join(d, "params.txt"))
    _xz(fi["stars"], os.path.join(d, "stars.txt.xz"))
    pf, sf = os.path.join(d, "params.txt"), fi["stars"]
    thetas = [np.asarray(fi["theta"])]
    if k == 2:
        thetas += [np.asarray(t) for t in m["thetas"][:4]]
    jobs = [(pf, sf, t, 0, 1) for t in thetas]
    nslices = 8 if k == 1 else 0
    jobs += [(pf, sf, thetas[0], r, nslices) for r in range(nslices)]
    t0 = time.time()
    res = _run(jobs)
    full = res[: len(thetas)]
    out = {"config": k, "n_stars": fi["n_stars"], "evaluations": full, "slices": res[len(thetas):],
           "wall_s": round(time.time() - t0, 1)}
    with open(os.path.join(d, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    for r in full:
        print(f"config{k}", r["likelihood"], r["wall_s"], "s", flush=True)


LARGE = {"86": ("86", "86", TEST_86), "12": ("12", "12", PARAM_SET1), "79": ("79", "79", TEST_79),
         # number_parameters 4 over seven background values: the aux a, b, c
         # are read from the file, the theta is the plain test's
         "79-aux": ("79-aux", "79", TEST_79),
         "86-aux": ("86-aux", "86", TEST_86[:2] + AUX_ABC + TEST_86[2:]),
         "11-aux": ("11-aux", "11", PARAM_SET1[:2] + AUX_ABC + PARAM_SET1[2:]),
         "12-aux": ("12-aux", "12", PARAM_SET1[:2] + AUX_ABC + PARAM_SET1[2:])}


def make_large(fid, nranks=8):
    import subprocess
    pname, sname, theta = LARGE[fid]
    d = os.path.join(HERE, "reference_large", fid)
    os.makedirs(d, exist_ok=True)
    pf = os.path.join(d, "params.txt")
    shutil.copyfile(os.path.join(REF_TESTS, f"astronomy_parameters-{pname}.txt"), pf)
    sf = os.path.join(REF_TESTS, f"stars-{sname}.txt")
    t0 = time.time()
    ranks = _run([(pf, sf, theta, r, nranks) for r in range(nranks)])
    S = len(ranks[0]["stream_integrals"])
    # integral_compose: plain sums in rank order
    ints = [0.0] * (1 + S)
    areas = [[0.0] * (1 + S) for _ in ranks[0]["area_integrals"]]
    for r in ranks:
        row = [r["background_integral"]] + r["stream_integrals"]
        for k in range(1 + S):
            ints[k] += row[k]
        for a, ar in enumerate(r["area_integrals"]):
            for k in range(1 + S):
                areas[a][k] += ar[k]
    ints = [float(x) for x in ints]
    areas = [[float(x) for x in a] for a in areas]
    out = subprocess.run([orc.REF_BIN, "-a", pf, "-p", sf, "-I", ",".join(repr(x) for x in ints),
                          *[repr(float(x)) for x in theta]], capture_output=True, text=True, check=True).stdout
    kv = dict(l.split(" ", 1) for l in out.strip().splitlines())
    g = {"background_integral": ints[0], "stream_integrals": ints[1:], "area_integrals": areas,
         "prob_sum": float(kv["prob_sum"]), "num_zero": int(kv["num_zero"]),
         "likelihood": float(kv["search_likelihood"]), "theta": [float(x) for x in theta],
         "method": f"the reference's distributed evaluation over {nranks} ranks (integral_compose, then "
                   f"calculate_likelihood over the whole catalogue)",
         "params_file": f"tests/astronomy_parameters-{pname}.txt", "stars_file": f"tests/stars-{sname}.txt",
         "stars_xz": f"reference/{sname}/stars.txt.xz", "rank_wall_s": [r["wall_s"] for r in ranks],
         "wall_s": round(time.time() - t0, 1)}
    with open(os.path.join(d, "golden.json"), "w") as f:
        json.dump(g, f, indent=1)
    print("large", fid, g["likelihood"], g["wall_s"], "s", flush=True)


def relikelihood(fid):
    """Recompute a large fixture's likelihood step from its stored composed
    integrals (the reference's calculate_likelihood against them)."""
    import subprocess
    pname, sname, theta = LARGE[fid]
    d = os.path.join(HERE, "reference_large", fid)
    g = json.load(open(os.path.join(d, "golden.json")))
    ints = [float(g["background_integral"])] + [float(x) for x in g["stream_integrals"]]
    out = subprocess.run([orc.REF_BIN, "-a", os.path.join(d, "params.txt"), "-p",
                          os.path.join(REF_TESTS, f"stars-{sname}.txt"), "-I", ",".join(repr(x) for x in ints),
                          *[repr(float(x)) for x in theta]], capture_output=True, text=True, check=True).stdout
    kv = dict(l.split(" ", 1) for l in out.strip().splitlines())
    g["prob_sum"], g["num_zero"] = float(kv["prob_sum"]), int(kv["num_zero"])
    g["likelihood"] = float(kv["search_likelihood"])
    with open(os.path.join(d, "golden.json"), "w") as f:
        json.dump(g, f, indent=1)
    print("large", fid, g["likelihood"], flush=True)


def make_slices():
    jobs, where = [], []
    for name in ("config0", "cut_area"):
        d = os.path.join(HERE, "cases", name)
        g = json.load(open(os.path.join(d, "golden.json")))
        for r in range(3):
            jobs.append((os.path.join(d, "params.txt"), os.path.join(d, "stars.txt"), g["theta"], r, 3))
            where.append(d)
    res = _run(jobs)
    for name in ("config0", "cut_area"):
        d = os.path.join(HERE, "cases", name)
        with open(os.path.join(d, "golden_slices.json"), "w") as f:
            json.dump([r for r, w in zip(res, where) if w == d], f, indent=1)
        print(name, "slices written", flush=True)


def main():
    orc.build(reference=True)
    if not orc.reference_available():
        sys.exit("the reference sources are needed to regenerate these goldens")
    work = os.environ.get("MWSEP_GOLDEN_WORK", os.path.join(REPO, "_work", "golden_data"))
    args = sys.argv[1:]
    if "--fixtures" in args:
        make_fixtures()
    if "--slices" in args:
        make_slices()
    for i, a in enumerate(args):
        if a == "--config":
            make_config(int(args[i + 1]), work)
        if a == "--large":
            make_large(args[i + 1])
        if a == "--relikelihood":
            relikelihood(args[i + 1])


if __name__ == "__main__":
    main()
