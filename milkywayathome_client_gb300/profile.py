"""Run a few evaluations of a benchmark workload, for profilers.

    python -m milkywayathome_client_gb300.profile --config 1 --precision mixed --evals 2

Prints the per-phase device times of each evaluation.  Used as the target of
ncu captures (one kernel, a couple of launches).
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
    ap.add_argument("--precision", choices=["plain", "mixed"], default="mixed")
    ap.add_argument("--evals", type=int, default=2)
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--data-dir", default=os.path.join(tempfile.gettempdir(), "mwsep_profile_data"))
    a = ap.parse_args()
    N.lib(build_if_missing=True)
    m = syn.materialise(a.config, a.data_dir)
    f = m["files"][0]
    prec = N.MWSEP_MIXED_F32 if a.precision == "mixed" else N.MWSEP_PLAIN_F64
    with Context(a.device) as ctx:
        ctx.set_problem(AstronomyParameters.read(f["params"]))
        ctx.set_stars(StarPoints.read(f["stars"]))
        for i in range(a.evals):
            if a.batch > 1:
                import numpy as np
                thetas = m.get("thetas")
                if thetas is None or len(thetas) < a.batch:
                    thetas = np.tile(f["theta"], (a.batch, 1))
                r = ctx.evaluate_batch(thetas[: a.batch], prec)[0]
            else:
                r = ctx.evaluate(f["theta"], prec)
            print(f"eval {i}: logL {r.likelihood:.15f} {ctx.last_timings()}", flush=True)


if __name__ == "__main__":
    main()
