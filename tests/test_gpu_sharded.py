"""The sharded evaluation on the GPU: the two per-rank steps of the
reference's distributed client (integral_f and likelihood_f,
cpu/astronomy_worker.c:33-121) and their composition (integral_compose,
likelihood_compose, :67-143).

* The phases run apart give the bits of the same phases of one evaluation.
* The worker entries mwsep_integral_f / mwsep_likelihood_f on a 3-way split
  of cut_area (two areas) against the reference's own sliced integrals, and
  the composed log-likelihood against the reference's whole evaluation.
* Two ranks (gloo processes sharing this GPU; each launches only its own
  kernels, the collectives are host-side sums) evaluate config0 sharded,
  within 1e-12 of the reference's whole evaluation.
"""
import json
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from conftest import CASES, REPO, load_case

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return abs(a - b) / abs(b) if b else abs(a)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_phases_apart_equal_one_evaluation(gpu_ctx, precision):
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case("cut_area")
    gpu_ctx.set_problem(mw.AstronomyParameters.read(pf))
    gpu_ctx.set_stars(mw.StarPoints.read(sf))
    whole = gpu_ctx.evaluate(g["theta"], precision)
    ints = gpu_ctx.integrals(g["theta"], precision)
    assert ints.integrals == whole.integrals and ints.area_integrals == whole.area_integrals
    assert np.isnan(ints.likelihood)
    lk = gpu_ctx.likelihood(g["theta"], whole.integrals, precision)
    assert lk.likelihood == whole.likelihood and lk.prob_sum == whole.prob_sum
    assert lk.num_zero == whole.num_zero and lk.integrals == whole.integrals


def test_worker_entries_match_reference_slices(built_library):
    """integral_f per rank against the reference's sliced integrals;
    likelihood_f per rank against the composed integrals; the composition
    against the reference's whole evaluation."""
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import sharding
    pf, sf, whole = load_case("cut_area")
    with open(os.path.join(CASES, "cut_area", "golden_slices.json")) as f:
        slices = json.load(f)
    n = slices[0]["nranks"]
    ranks = []
    for g in slices:
        ap, sp = mw.AstronomyParameters.read(pf), mw.StarPoints.read(sf)
        ap.split(g["rank"], n)
        sp.split(g["rank"], n)
        es = mw.EvaluationState(ap, sp)
        res = mw.integral_f(g["theta"], ap, es, sp)
        want = np.asarray(g["area_integrals"][0]) - np.sum(g["area_integrals"][1:], axis=0)
        for x, y in zip(res, want):
            assert _rel(x, y) <= 1e-12, (g["rank"], x, y)
        for got, w in zip(es.area_integrals, g["area_integrals"]):
            for x, y in zip(got, w):
                assert _rel(x, y) <= 1e-12, (g["rank"], x, y)
        ranks.append((ap, sp, es, res))
    composed = sharding.integral_compose([r[3] for r in ranks])
    for x, y in zip(composed, [whole["background_integral"]] + whole["stream_integrals"]):
        assert _rel(x, y) <= 1e-12, (x, y)
    lks = [mw.likelihood_f(composed, ap, es, sp) for ap, sp, es, _ in ranks]
    total = mw.StarPoints.read(sf).number_stars
    assert abs(sharding.likelihood_compose(lks, total) - whole["likelihood"]) <= 1e-12


_RANK = textwrap.dedent("""
    import json, os, sys
    sys.path.insert(0, {repo!r})
    import torch.distributed as dist
    from milkywayathome_client_gb300 import sharding
    dist.init_process_group("gloo", rank=int(os.environ["RANK"]), world_size=int(os.environ["WORLD_SIZE"]))
    theta = json.loads(os.environ["THETA"])
    out = {{}}
    for prec in (0, 2, 1):
        ints, ll = sharding.evaluate_sharded(os.environ["PF"], os.environ["SF"], theta, prec)
        out[str(prec)] = {{"integrals": [float(x) for x in ints], "likelihood": ll}}
    dist.destroy_process_group()
    print(json.dumps(out))
""")


def test_two_ranks_compose_the_whole_evaluation(built_library, tmp_path):
    """Two gloo ranks, each integrating half the cells and evaluating half
    the stars on this GPU, against the reference's whole evaluation: the
    plain and double-float forms within 1e-12, the compensated form within
    1e-7 on the log-likelihood."""
    import socket
    pf, sf, g = load_case("config0")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", PF=pf, SF=sf,
               THETA=json.dumps(g["theta"]))
    code = _RANK.format(repo=REPO)
    procs = [subprocess.Popen([sys.executable, "-c", code], env=dict(env, RANK=str(r)), stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=600)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    assert outs[0] == outs[1]  # every rank holds the same composed values
    want = [g["background_integral"]] + g["stream_integrals"]
    for prec, rel, dl in (("0", 1e-12, 1e-12), ("2", 1e-12, 1e-12), ("1", 2e-7, 1e-7)):
        r = outs[0][prec]
        for x, y in zip(r["integrals"], want):
            assert _rel(x, y) <= rel, (prec, x, y)
        assert abs(r["likelihood"] - g["likelihood"]) <= dl, (prec, r["likelihood"], g["likelihood"])
