"""The debug build with device-side index checks (-DMWSEP_DEVICE_CHECKS=1):
built into a temporary directory and run, in a child process, over small
cases through every device entry point (single and batched evaluations in
both forms, engine requests over several wedges, separation).  No
instrumented index may be out of range, and the results must equal the
normal build's."""
import json
import os
import subprocess
import sys

import pytest

from conftest import REPO, load_case

pytestmark = pytest.mark.gpu

CASES = ["basic_1stream", "cut_area", "six_streams", "aux_profile", "general_alpha_delta", "ragged_sizes",
         "single_cell_single_star"]

CHILD = r'''
import ctypes as C, json, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import milkywayathome_client_gb300 as mw
from milkywayathome_client_gb300 import native as N
cases = json.loads(sys.argv[2])
out = {}
en, fail, first = C.c_int(), C.c_ulonglong(), C.c_ulonglong()
with mw.Context(0) as ctx:
    wids = []
    for name, pf, sf, theta in cases:
        ap, sp = mw.AstronomyParameters.read(pf), mw.StarPoints.read(sf)
        ctx.set_problem(ap); ctx.set_stars(sp)
        r = [ctx.evaluate(theta, p).likelihood for p in (0, 1)]
        b = [x.likelihood for x in ctx.evaluate_batch([theta, theta], 1)]
        sep = ctx.separation(theta, seed=3)
        out[name] = {"single": r, "batch": b, "sep": float(np.sum(sep["sprob"])) if sep["sprob"].size else 0.0}
        wids.append((ctx.add_wedge(ap, sp), theta))
    for p in (0, 1):
        res = ctx.evaluate_requests([(w, t) for w, t in wids], p)
        for (name, _, _, _), x in zip(cases, res):
            out[name]["engine%d" % p] = x.likelihood
N.check(N.lib().mwsep_device_checks(0, C.byref(en), C.byref(fail), C.byref(first)))
print(json.dumps({"enabled": en.value, "failures": fail.value, "first": first.value, "out": out}))
'''


def _run(lib, cases):
    env = dict(os.environ)
    if lib:
        env["MWSEP_LIBRARY"] = lib
    r = subprocess.run([sys.executable, "-c", CHILD, REPO, json.dumps(cases)], capture_output=True, text=True,
                       env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_device_checks_build(built_library, tmp_path):
    from milkywayathome_client_gb300 import build
    lib = str(tmp_path / "libmwsep_gb300.so")
    build.build(force=True, extra_flags=["-DMWSEP_DEVICE_CHECKS=1"], lib_path=lib, build_dir=str(tmp_path / "b"))
    cases = []
    for name in CASES:
        pf, sf, g = load_case(name)
        cases.append((name, pf, sf, g["theta"]))
    checked = _run(lib, cases)
    plain = _run(None, cases)
    assert checked["enabled"] == 1 and plain["enabled"] == 0
    assert checked["failures"] == 0, hex(checked["first"])
    assert checked["out"] == plain["out"]
