"""Run a few evaluations of a benchmark workload, for profilers.

    python -m milkywayathome_client_gb300.profile --config 1 --precision mixed --evals 2
    python -m milkywayathome_client_gb300.profile --config 2 --batch 256 [--engine]

Prints the per-phase device times of each evaluation (or batch).  Used as
the target of ncu captures (one kernel, a couple of launches).  --batch B
evaluates B parameter vectors per call: on the single-wedge path
(gridDim.y = B) or, with --engine, as one engine batch of requests.
"""
from __future__ import annotations

import argparse
import os
import tempfile

from . import native as N
from . import synthetic as syn
from .separation import AstronomyParameters, Context, StarPoints


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--precision", choices=["plain", "mixed", "df"], default="mixed")
    ap.add_argument("--evals", type=int, default=2)
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--engine", action="store_true")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--data-dir", default=os.path.join(tempfile.gettempdir(), "mwsep_profile_data"))
    a = ap.parse_args()
    N.lib(build_if_missing=True)
    m = syn.materialise(a.config, a.data_dir)
    f = m["files"][0]
    prec = {"mixed": N.MWSEP_MIXED_F32, "plain": N.MWSEP_PLAIN_F64, "df": N.MWSEP_PLAIN_DF}[a.precision]
    import numpy as np
    thetas = m.get("thetas")
    if thetas is None or len(thetas) < a.batch:
        thetas = np.tile(f["theta"], (a.batch, 1))
    thetas = thetas[: a.batch]
    with Context(a.device) as ctx:
        ap, sp = AstronomyParameters.read(f["params"]), StarPoints.read(f["stars"])
        ctx.set_problem(ap)
        ctx.set_stars(sp)
        wid = ctx.add_wedge(ap, sp) if a.engine else None
        for i in range(a.evals):
            if a.engine:
                r = ctx.evaluate_requests([(wid, t) for t in thetas], prec)[0]
            elif a.batch > 1:
                r = ctx.evaluate_batch(thetas, prec)[0]
            else:
                r = ctx.evaluate(f["theta"], prec)
            print(f"eval {i}: logL {r.likelihood:.15f} {ctx.last_timings()}", flush=True)


if __name__ == "__main__":
    main()
