"""Serving benchmark: Poisson arrivals over resident wedges.

    python -m milkywayathome_client_gb300.serve_bench --rates 50,200,800 --seconds 4 --precision mixed|plain|df

The wedges are those of the mixed-size workload (6 seeded synthetic wedges,
log-uniform sizes; synthetic.config(3)), all resident at once; each arrival
picks a wedge with probability proportional to its star count and perturbs
that wedge's parameter vector.  For every rate the server is fed for
--seconds of arrivals, then drained; the line reports p50/p99 latency
(submit -> result) and completed evaluations per second.
"""
from __future__ import annotations

import argparse
import json
import os
import tempfile
import time

import numpy as np

from . import native as N
from . import synthetic as syn
from .separation import AstronomyParameters, Context, Server, StarPoints


HBM_BUDGET_BYTES = 160 * 10 ** 9  # the device-memory budget requests are admitted against


def run(rates, seconds, precision, lanes, max_batch, data_dir, autotune=True, star_scale=1.0, seed=0,
        ctx=None, wedges=None, target_batch_ms=0.0, max_queued=0, hbm_budget=HBM_BUDGET_BYTES):
    """Feed a server Poisson arrivals at each rate for `seconds`, drain, and
    report latency, throughput and admission.  The wedges' resident bytes
    come out of hbm_budget first; the rest is split evenly over the lanes'
    batch buffers (0: no budget)."""
    own = ctx is None
    if own:
        ctx = Context(0)
        m = syn.materialise(3, data_dir, star_scale=star_scale)
        wedges = []
        for f in m["files"]:
            wid = ctx.add_wedge(AstronomyParameters.read(f["params"]), StarPoints.read(f["stars"]))
            wedges.append((wid, f["theta"], f["n_stars"]))
        if autotune:
            for wid, _, _ in wedges:
                ctx.autotune(wid, precision)
    stars = np.array([w[2] for w in wedges], float)
    p = stars / stars.sum()
    out = []
    lane_bytes = 0
    if hbm_budget:
        resident = sum(ctx.wedge_bytes(w[0]) for w in wedges)
        lane_bytes = max(1, (hbm_budget - resident) // lanes)
    with Server(ctx, lanes=lanes, max_batch=max_batch, lane_hbm_bytes=lane_bytes, target_batch_ms=target_batch_ms,
                max_queued=max_queued) as srv:
        # warm-up: one request per wedge (captures the lanes' graphs)
        for wid, th, _ in wedges:
            srv.wait(srv.submit(wid, th, precision), 600)
        for rate in rates:
            rng = np.random.default_rng(seed + int(rate))
            srv.reset_stats()
            ids = []
            t0 = time.perf_counter()
            t_next = t0
            while True:
                t_next += rng.exponential(1.0 / rate)
                if t_next - t0 > seconds:
                    break
                delay = t_next - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                k = rng.choice(len(wedges), p=p)
                wid, th, _ = wedges[k]
                theta = np.asarray(th) * (1.0 + 0.001 * rng.standard_normal(len(th)))
                try:
                    ids.append(srv.submit(wid, theta, precision))
                except N.MwsepError as e:
                    if e.status != N.MWSEP_ERR_BUSY:
                        raise
            for i in ids:
                srv.wait(i, 3600)
            st = srv.stats()
            out.append({"rate_req_s": rate, "arrivals": len(ids) + st["refused"], "accepted": len(ids),
                        "refused": st["refused"], "p50_latency_s": st["p50_latency_s"],
                        "p99_latency_s": st["p99_latency_s"], "evals_per_s": st["evals_per_s"],
                        "mean_batch": st["mean_batch"], "batches": st["batches"], "max_queue": st["max_queue"]})
    if own:
        ctx.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rates", default="50,200,800")
    ap.add_argument("--seconds", type=float, default=4.0)
    ap.add_argument("--precision", choices=["plain", "mixed", "df"], default="mixed")
    ap.add_argument("--lanes", type=int, default=2)
    ap.add_argument("--max-batch", type=int, default=256)
    ap.add_argument("--star-scale", type=float, default=1.0)
    ap.add_argument("--target-batch-ms", type=float, default=0.0)
    ap.add_argument("--max-queued", type=int, default=0)
    ap.add_argument("--data-dir", default=os.path.join(tempfile.gettempdir(), "mwsep_serve_data"))
    a = ap.parse_args()
    prec = {"mixed": N.MWSEP_MIXED_F32, "plain": N.MWSEP_PLAIN_F64, "df": N.MWSEP_PLAIN_DF}[a.precision]
    rates = [float(x) for x in a.rates.split(",")]
    res = run(rates, a.seconds, prec, a.lanes, a.max_batch, a.data_dir, star_scale=a.star_scale,
              target_batch_ms=a.target_batch_ms, max_queued=a.max_queued)
    print(json.dumps({"precision": a.precision, "lanes": a.lanes, "results": res}))


if __name__ == "__main__":
    main()
