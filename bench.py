#!/usr/bin/env python
"""Separation-likelihood throughput on GB300: evaluations per second.

Workload: the full-size single evaluation (1600 x 640 x 140 cells, 120
convolution points, 3 streams, 100k stars; seeded synthetic wedge, see
milkywayathome_client_gb300/synthetic.py).  A step is one evaluation
(integrals over every cell + likelihood over every star).

  value      evaluations/s in the compensated-FP32 form with the wedge and
             catalogue resident in HBM (device time from CUDA events on the
             library's stream; L2 flushed between steps)
  plain_f64  the same for the plain FP64 drop-in form
  plain_double_float  the same for the double-float form (plain-form
             accuracy, 1e-12, computed in pairs of FP32 values)
  e2e        evaluations/s through the reference-facing EvalFunc C-ABI call
             (mwsep_evaluate_mixed) with host structs: every step uploads the
             catalogue, rebuilds the wedge and star tables, evaluates and
             reads the result back
  roofline   the dominant kernel (compensated integral) against the SFU
             throughput measured by the library's own pipe microbenchmark
  cpu_baseline  the reference CPU evaluator (or its C restatement where the
             reference is not compiled on this host) on a bounded slice of
             the same evaluation, all host cores
  extras     population_batch (256 parameter vectors of one wedge, one
             engine batch), mixed_size_batch (64 evaluations over 6 wedges
             of log-uniform sizes, per-wedge autotuned tiles, one engine
             batch replayed as a CUDA graph), serving (Poisson arrivals),
             catalogue_load (text vs binary catalogue)

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "evals/s mixed-FP32 vs plain FP64 at |dlogL|<=1e-7"
CONFIG_INDEX = 1
CPU_SLICES = 400  # the CPU baseline evaluates 1/400-slices of the workload


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the population-batch and serving measurements")
    ap.add_argument("--extras", default="population,mixed,serving,catalogue",
                    help="comma list of the extra measurements to run (population, mixed, serving, catalogue)")
    ap.add_argument("--workload", type=int, default=CONFIG_INDEX, choices=[0, 1, 2],
                    help="benchmark config of the single-evaluation steps (default 1, the full-size wedge; "
                         "0 and 2 are smaller wedges, for profiling runs)")
    ap.add_argument("--data-dir", default=os.path.join(tempfile.gettempdir(), "mwsep_bench_data"))
    return ap.parse_args()


GOLDEN = os.path.join(REPO, "tests", "golden")


def workload_files(idx, data_dir):
    """Parameter and star files of a benchmark config, with the reference's
    own outputs on them when the repository holds them: configs 1 and 2 from
    their committed inputs (tests/golden/scale, the reference CPU evaluator's
    goldens), config 0 from tests/golden/cases/config0.  Returns (files,
    golden evaluation or None)."""
    import json as _json
    import lzma
    from milkywayathome_client_gb300 import synthetic as syn
    src = {1: os.path.join(GOLDEN, "scale", "config1"), 2: os.path.join(GOLDEN, "scale", "config2"),
           0: os.path.join(GOLDEN, "cases", "config0")}[idx]
    gpath = os.path.join(src, "golden.json")
    if not os.path.exists(gpath):
        return [dict(syn.materialise(idx, data_dir)["files"][0])], None
    os.makedirs(data_dir, exist_ok=True)
    f = {"problem": syn.config(idx)["problems"][0]}
    g = _json.load(open(gpath))
    ev = g["evaluations"][0] if "evaluations" in g else g
    f["params"] = os.path.join(src, "params.txt")
    if os.path.exists(os.path.join(src, "stars.txt.xz")):
        out = os.path.join(data_dir, f"config{idx}_golden_stars.txt")
        if not os.path.exists(out):
            with lzma.open(os.path.join(src, "stars.txt.xz"), "rb") as a, open(out + ".part", "wb") as b:
                shutil.copyfileobj(a, b)
            os.replace(out + ".part", out)
        f["stars"] = out
    else:
        f["stars"] = os.path.join(src, "stars.txt")
    f["theta"] = ev["theta"]
    with open(f["stars"]) as fh:
        f["n_stars"] = int(fh.readline())
    return [f], ev


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=ws)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(ws, x):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_desc(files):
    f = files[0]
    p = f["problem"]
    a = p.areas[0]
    return {"workload": f"separation likelihood, one evaluation: {a.mu[2]}x{a.nu[2]}x{a.r[2]} (mu x nu x r) "
                        f"cells, convolve {p.convolve}, {len(p.streams)} streams, {f['n_stars']} stars",
            "mu_steps": a.mu[2], "nu_steps": a.nu[2], "r_steps": a.r[2], "convolve": p.convolve,
            "streams": len(p.streams), "stars": f["n_stars"], "wedge": p.wedge}


def points_per_eval(files):
    f = files[0]
    p = f["problem"]
    cells = p.cells()
    return cells * p.convolve, f["n_stars"] * p.convolve


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.fh = open(self.path, "w")
        self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader",
                                      "-lms", "200", "-i", str(self.device)], stdout=self.fh,
                                     stderr=subprocess.DEVNULL)
        time.sleep(0.3)

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                mx = float(parts[2].split()[0])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ CPU side
def cpu_ranks(n_procs, slices=CPU_SLICES):
    """The slices the CPU baseline times: n_procs ranks of `slices`, spread
    evenly over the linearised cell index and the catalogue (the cost of a
    slice depends on where it lies relative to the streams)."""
    return [(i * slices) // n_procs for i in range(n_procs)]


def cpu_sample(files, theta, n_procs, slices=CPU_SLICES):
    """Run n_procs concurrent slices (cpu_ranks) of the evaluation on the
    host and return (wall seconds, kind, binary)."""
    from oracle import oracle as orc
    ref_bin, port_bin = orc.REF_BIN, orc.ORACLE_BIN
    kind, binary = None, None
    f = files[0]
    args_theta = [repr(float(x)) for x in theta]
    for k, b in (("reference", ref_bin), ("port", port_bin)):
        if os.path.exists(b):
            try:
                r = subprocess.run([b, "-a", f["params"], "-p", f["stars"], "-r", "0", "-n", "100000",
                                    *args_theta], capture_output=True, timeout=60)
                if r.returncode == 0:
                    kind, binary = k, b
                    break
            except OSError:
                continue
    if binary is None:
        orc.build(reference=False)
        kind, binary = "port", port_bin
    t0 = time.perf_counter()
    procs = [subprocess.Popen([binary, "-a", f["params"], "-p", f["stars"], "-r", str(r), "-n", str(slices),
                               *args_theta], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
             for r in cpu_ranks(n_procs, slices)]
    rcs = [p.wait() for p in procs]
    wall = time.perf_counter() - t0
    if any(rcs):
        raise RuntimeError(f"CPU baseline slices failed: {rcs}")
    return wall, kind, binary


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference_arm(args, ws, rank):
    """--impl reference: the reference's CPU evaluator on the host cores."""
    if rank != 0:
        return
    files, _ = workload_files(args.workload, os.path.join(args.data_dir, "rank0"))
    theta = files[0]["theta"]
    n = min(host_cores(), 64)
    times = []
    kind = "port"
    for i in range(args.warmup + args.steps):
        wall, kind, _ = cpu_sample(files, theta, n)
        if i >= args.warmup:
            times.append(wall)
    t = sum(times) / len(times)
    value = (n / CPU_SLICES) / t
    sample = (f"{n} concurrent processes, each 1/{CPU_SLICES} of the evaluation (the reference's own "
              f"rank slicing of cells and stars), ranks {cpu_ranks(n)} of {CPU_SLICES} "
              f"({n}/{CPU_SLICES} of the evaluation) per step")
    cpu = {"value": value, "unit": "evals/s", "cores": n, "kind": kind, "sample": sample}
    out = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": workload_desc(files), "cpu_baseline": cpu,
           "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ GPU arm
def traffic_from_profiles(kernel_key):
    """dram bytes per launch recorded from an ncu capture (profiles/)."""
    path = os.path.join(REPO, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel_key and not line.startswith("#"):
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def run_gb300_arm(args, ws, rank, local):
    import ctypes as C
    import torch
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import native as N
    from milkywayathome_client_gb300 import synthetic as syn

    N.lib(build_if_missing=True)
    device = local
    torch.cuda.set_device(device)
    files, golden = workload_files(args.workload, os.path.join(args.data_dir, f"rank{rank}"))
    f = files[0]
    theta = f["theta"]
    S = len(f["problem"].streams)
    ap = mw.AstronomyParameters.read(f["params"])
    sp = mw.StarPoints.read(f["stars"])
    ctx = mw.Context(device)
    ctx.set_problem(ap)
    ctx.set_stars(sp)

    peaks = N.mwsep_pipe_peaks()
    N.check(N.lib().mwsep_measure_pipe_peaks(device, C.byref(peaks)), "pipe microbenchmark")

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{device}")

    def step(precision):
        flush.zero_()
        torch.cuda.synchronize(device)
        r = ctx.evaluate(theta, precision)
        t = ctx.last_timings()
        return r, t, ctx.last_launches()

    # compensated FP32: warm-up then K timed steps
    for _ in range(max(args.warmup, 3)):
        step(N.MWSEP_MIXED_F32)
    clocks = ClockSampler(device)
    barrier(ws)
    torch.cuda.synchronize(device)
    clocks.start()
    dev_ms, integ_ms, launches = [], [], 0
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        r32, t, nl = step(N.MWSEP_MIXED_F32)
        dev_ms.append(t["total_ms"])
        integ_ms.append(t["integral_ms"])
        launches += nl
    torch.cuda.synchronize(device)
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    barrier(ws)
    total_ms = allreduce_max(ws, sum(dev_ms))
    ms_per_step = total_ms / args.steps
    value = ws * args.steps / (total_ms * 1e-3)

    # plain FP64 (the drop-in form) for the headline comparison
    step(N.MWSEP_PLAIN_F64)
    f64_ms = []
    for _ in range(args.plain_steps):
        r64, t, _ = step(N.MWSEP_PLAIN_F64)
        f64_ms.append(t["total_ms"])
    f64_ms_step = allreduce_max(ws, sum(f64_ms)) / args.plain_steps
    plain_value = ws / (f64_ms_step * 1e-3)

    # the double-float form: plain-form accuracy (1e-12) on the FP32 pipes
    step(N.MWSEP_PLAIN_DF)
    df_ms = []
    for _ in range(args.plain_steps):
        rdf, t, _ = step(N.MWSEP_PLAIN_DF)
        df_ms.append(t["total_ms"])
    df_ms_step = allreduce_max(ws, sum(df_ms)) / args.plain_steps
    double_float = {"value": ws / (df_ms_step * 1e-3), "unit": "evals/s", "ms_per_step": df_ms_step,
                    "dtype": "f32 pairs (double-float)",
                    "speedup_vs_plain_f64": f64_ms_step / df_ms_step,
                    "dlogL_vs_plain_f64": rdf.likelihood - r64.likelihood,
                    "max_integral_rel_err_vs_plain_f64": max(abs(a - b) / abs(b) if b else 0.0
                                                             for a, b in zip(rdf.integrals, r64.integrals))}

    # e2e through the EvalFunc C ABI with host buffers
    es = mw.EvaluationState(ap, sp)
    mw.evaluate_mixed(theta, ap, es, sp)  # warm-up (creates the library's default context)
    e2e_t = []
    h2d = C.c_size_t()
    d2h = C.c_size_t()
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        v = mw.evaluate_mixed(theta, ap, es, sp)
        e2e_t.append(time.perf_counter() - t0)
    N.lib().mwsep_evalfunc_transfer_bytes(C.byref(h2d), C.byref(d2h))
    e2e_step = allreduce_max(ws, sum(e2e_t)) / args.e2e_steps
    e2e_value = ws / e2e_step
    e2e_logl = v - 3.0
    # the double-float form through its EvalFunc entry (mwsep_evaluate_df)
    es_df = mw.EvaluationState(ap, sp)
    mw.evaluate_df(theta, ap, es_df, sp)
    t0 = time.perf_counter()
    mw.evaluate_df(theta, ap, es_df, sp)
    double_float["e2e"] = {"value": ws / allreduce_max(ws, time.perf_counter() - t0), "unit": "evals/s",
                           "api": "mwsep_evaluate_df (EvalFunc, host structs)"}

    # roofline of the dominant kernel (the compensated integral, packed warp
    # tiles).  Per convolution point it issues 10.5 + 4S FP32 lane-ops
    # (t 2, halo quadratic 2, rg + r0 1, cube 2, the four-point fraction
    # sum 3.5; per stream offset, two-FMA exponent, accumulate) and 1.25 + S
    # SFU ops (rsqrt, a quarter rcp, S ex2).  Its
    # peak is the point rate of the slower of the two pipes at the rates the
    # library's microbenchmark measures on this GPU.
    cell_pts, star_pts = points_per_eval(files)
    fp32_ops = 10.5 + 4 * S
    sfu_s_per_point = 1.0 / (peaks.rsqrt_gops * 1e9) + 0.25 / (peaks.rcp_gops * 1e9) + S / (peaks.ex2_gops * 1e9)
    fma_s_per_point = fp32_ops / (peaks.fp32_fma_tflops * 1e12 / 2.0)
    peak = 1.0 / max(sfu_s_per_point, fma_s_per_point) / 1e9
    integ_s = statistics.median(integ_ms) * 1e-3
    achieved = cell_pts / integ_s / 1e9
    traffic = traffic_from_profiles("integral_f32w_config1")
    roofline = {"bound": "fma+sfu", "achieved": achieved, "peak": peak, "unit": "Gpoint/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": "integral_f32w_dyn_kernel (packed warp tiles, tile counter)",
                "peak_source": "measured (project pipe microbenchmark, mwsep_measure_pipe_peaks): FP32 FMA, "
                               "rsqrt, rcp and ex2 rates, at this kernel's per-point op mix",
                "work_per_point": f"{fp32_ops} FP32 lane-ops + {1.25 + S} SFU ops",
                "binding_pipe": "fma" if fma_s_per_point >= sfu_s_per_point else "sfu",
                "points_per_launch": cell_pts}
    # the same throughput in the reference's own operation count: F(S) = 18 + 23 S
    # flops per density point (every +, -, x, /, sqrt, exp counted once)
    F = 18 + 23 * S
    pts_eval = cell_pts + star_pts
    algorithmic = {"flops_per_point": F, "points_per_eval": pts_eval,
                   "mixed_tflops": pts_eval * F * value / 1e12,
                   "plain_f64_tflops": pts_eval * F * plain_value / 1e12,
                   "note": "reference operation count; divide, sqrt and exp expand to many pipe "
                           "instructions, so the pipe roofline above is the binding one"}

    out = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": dict(workload_desc(files), l2="flushed between steps (256 MB write)",
                       parallelism="replicas" if ws > 1 else "single GPU"),
        "impl": "gb300",
        "plain_f64": {"value": plain_value, "unit": "evals/s", "ms_per_step": f64_ms_step, "dtype": "f64"},
        "plain_double_float": double_float,
        "speedup_mixed_vs_plain": value / plain_value,
        "dlogL_mixed_vs_plain": r32.likelihood - r64.likelihood,
        "integral_rel_err_mixed_vs_plain": [(a - b) / b if b else 0.0 for a, b in zip(r32.integrals,
                                                                                    r64.integrals)],
        "likelihood": {"plain_f64": r64.likelihood, "mixed_f32": r32.likelihood, "e2e_mixed": e2e_logl},
        "points_per_s": {"integral": ws * cell_pts / (ms_per_step * 1e-3),
                         "likelihood": ws * star_pts / (ms_per_step * 1e-3)},
        "e2e": {"value": e2e_value, "unit": "evals/s", "h2d_bytes_per_step": h2d.value,
                "d2h_bytes_per_step": d2h.value, "api": "mwsep_evaluate_mixed (EvalFunc, host structs)"},
        "gpu_launches": launches,
        "roofline": roofline,
        "roofline_algorithmic": algorithmic,
        "pipe_peaks": {"fp64_tflops": peaks.fp64_fma_tflops, "fp32_tflops": peaks.fp32_fma_tflops,
                       "ex2_gops": peaks.ex2_gops, "rsqrt_gops": peaks.rsqrt_gops, "rcp_gops": peaks.rcp_gops},
        "wall_s_timed": wall,
    }
    if golden is not None:
        # each form against the reference CPU evaluator's own result on these inputs
        def err(r):
            return {"dlogL": r.likelihood - golden["likelihood"],
                    "max_integral_rel_err": max(abs(a - b) / abs(b) if b else 0.0 for g_area, w_area in
                                                zip(r.area_integrals, golden["area_integrals"])
                                                for a, b in zip(g_area, w_area))}
        out["accuracy_vs_reference"] = {
            "golden": f"the reference CPU evaluator's own result on these inputs (tests/golden, config "
                      f"{args.workload})",
            "mixed_f32": err(r32), "plain_f64": err(r64), "double_float": err(rdf)}
        out["dlogL_mixed_vs_oracle"] = r32.likelihood - golden["likelihood"]
    if clk:
        out["clocks"] = clk
    extras = set() if args.no_extras else {e.strip() for e in args.extras.split(",") if e.strip()}
    if rank == 0 and extras:
        ctx.close()
        ctx = None
        if "population" in extras:
            out["population_batch"] = population_batch(args)
        if "mixed" in extras:
            out["mixed_size_batch"] = mixed_size_batch(args)
        if "serving" in extras:
            out["serving"] = serving(args)
        if "catalogue" in extras:
            out["catalogue_load"] = catalogue_load(args, files)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        n = min(host_cores(), 64)
        cw, kind, _ = cpu_sample(files, theta, n)
        cv = (n / CPU_SLICES) / cw
        out["cpu_baseline"] = {"value": cv, "unit": "evals/s", "cores": n, "kind": kind,
                               "sample": f"{n} concurrent 1/{CPU_SLICES} slices of the evaluation "
                                         f"(reference rank slicing of cells and stars), ranks "
                                         f"{cpu_ranks(n)} of {CPU_SLICES} spread over the index, "
                                         f"{cw:.1f} s wall"}
    if ctx is not None:
        ctx.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


def population_batch(args):
    """256 parameter vectors on one wedge (400 x 160 x 140, convolve 60,
    3 streams, 50k stars) evaluated as one engine batch, compensated FP32."""
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import synthetic as syn
    m = syn.materialise(2, os.path.join(args.data_dir, "population"))
    f = m["files"][0]
    thetas = m["thetas"]
    with mw.Context(0) as ctx:
        wid = ctx.add_wedge(mw.AstronomyParameters.read(f["params"]), mw.StarPoints.read(f["stars"]))
        ctx.autotune(wid, mw.MWSEP_MIXED_F32)
        reqs = [(wid, t) for t in thetas]
        ctx.evaluate_requests(reqs, mw.MWSEP_MIXED_F32)
        times = []
        for _ in range(3):
            res = ctx.evaluate_requests(reqs, mw.MWSEP_MIXED_F32)
            times.append(ctx.last_timings()["total_ms"])
        launches = ctx.last_launches()
        plain = ctx.evaluate_requests(reqs[:4], mw.MWSEP_PLAIN_F64)
        plain_ms = ctx.last_timings()["total_ms"]
        # the plain form's accuracy in double-float: the whole population, one batch
        ctx.evaluate_requests(reqs[:8], mw.MWSEP_PLAIN_DF)
        dfres = ctx.evaluate_requests(reqs, mw.MWSEP_PLAIN_DF)
        df_ms = ctx.last_timings()["total_ms"]
        # the errors() consumer: a finite-difference Hessian (2P^2+1 points) as engine batches
        step = mw.AstronomyParameters.read(f["params"]).step()
        P = len(step)
        t0 = time.perf_counter()
        ctx.hessian(wid, thetas[0], step, mw.MWSEP_MIXED_F32)
        hess_s = time.perf_counter() - t0
    ms = statistics.median(times)
    return {"workload": "256 parameter vectors, 400x160x140 cells, convolve 60, 3 streams, 50k stars",
            "value": len(thetas) / (ms * 1e-3), "unit": "evals/s", "ms_per_batch": ms,
            "launches_per_batch": launches, "graph": True,
            "plain_f64_evals_per_s": 4 / (plain_ms * 1e-3),
            "max_dlogL_mixed_vs_plain": max(abs(a.likelihood - b.likelihood) for a, b in zip(res[:4], plain)),
            "double_float_evals_per_s": len(reqs) / (df_ms * 1e-3),
            "max_dlogL_double_float_vs_plain": max(abs(a.likelihood - b.likelihood)
                                                   for a, b in zip(dfres[:4], plain)),
            "hessian": {"parameters": P, "evaluations": 2 * P * P + 1, "seconds": hess_s,
                        "evals_per_s": (2 * P * P + 1) / hess_s, "precision": "mixed"}}


def catalogue_load(args, files):
    """Making the 100k-star catalogue resident: the reference's text file
    (parse + upload + star tables) against the binary catalogue (map +
    upload + star tables)."""
    import milkywayathome_client_gb300 as mw
    f = files[0]
    binp = os.path.join(args.data_dir, "catalogue.mwsb")
    mw.StarPoints.read(f["stars"]).write_binary(binp)
    out = {}
    with mw.Context(0) as ctx:
        ctx.set_problem(mw.AstronomyParameters.read(f["params"]))
        for kind, path in (("text", f["stars"]), ("binary", binp), ("text", f["stars"]), ("binary", binp)):
            t0 = time.perf_counter()
            ctx.set_stars_file(path)
            out[kind] = (time.perf_counter() - t0) * 1e3
    return {"stars": f["n_stars"], "text_ms": out["text"], "binary_ms": out["binary"],
            "speedup": out["text"] / out["binary"]}


def mixed_size_batch(args):
    """64 evaluations spread over the 6 mixed-size wedges (log-uniform sizes,
    the serving wedges), each wedge's tile shape from the autotuner, one
    engine batch replayed as a CUDA graph, compensated FP32; and one
    evaluation per wedge in the plain FP64 and double-float forms, for their
    rates and the compensated form's error."""
    import numpy as np
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import synthetic as syn
    m = syn.materialise(3, os.path.join(args.data_dir, "serving"))
    rng = np.random.default_rng(3)
    with mw.Context(0) as ctx:
        wedges = []
        for f in m["files"]:
            wid = ctx.add_wedge(mw.AstronomyParameters.read(f["params"]), mw.StarPoints.read(f["stars"]))
            wedges.append((wid, np.asarray(f["theta"], dtype=np.float64), f["n_stars"]))
        for wid, _, _ in wedges:
            ctx.autotune(wid, mw.MWSEP_MIXED_F32)
        p = np.array([w[2] for w in wedges], float)
        p /= p.sum()
        reqs = []
        for _ in range(64):
            wid, th, _ = wedges[rng.choice(len(wedges), p=p)]
            reqs.append((wid, th * (1.0 + 0.002 * rng.standard_normal(th.size))))
        ctx.evaluate_requests(reqs, mw.MWSEP_MIXED_F32)  # graph capture
        times = []
        for _ in range(3):
            ctx.evaluate_requests(reqs, mw.MWSEP_MIXED_F32)
            times.append(ctx.last_timings()["total_ms"])
        sweep = [(wid, th) for wid, th, _ in wedges]
        mixed = ctx.evaluate_requests(sweep, mw.MWSEP_MIXED_F32)
        rates = {}
        out = {}
        for name, prec in (("plain_f64", mw.MWSEP_PLAIN_F64), ("double_float_untuned", mw.MWSEP_PLAIN_DF)):
            out[name] = ctx.evaluate_requests(sweep, prec)
            rates[name] = len(sweep) / (ctx.last_timings()["total_ms"] * 1e-3)
        for wid, _, _ in wedges:
            ctx.autotune(wid, mw.MWSEP_PLAIN_DF)
        out["double_float"] = ctx.evaluate_requests(sweep, mw.MWSEP_PLAIN_DF)
        rates["double_float"] = len(sweep) / (ctx.last_timings()["total_ms"] * 1e-3)
    ms = statistics.median(times)
    return {"workload": "64 evaluations over 6 wedges (mu 200-1600, nu 80-640, r 70-700, convolve 30-120, "
                        "1-4 streams, 20k-200k stars), wedge chosen by star count",
            "value": len(reqs) / (ms * 1e-3), "unit": "evals/s", "ms_per_batch": ms, "graph": True,
            "autotuned": True,
            "plain_f64_evals_per_s": rates["plain_f64"], "double_float_evals_per_s": rates["double_float"],
            "double_float_untuned_evals_per_s": rates["double_float_untuned"],
            "max_dlogL_mixed_vs_plain": max(abs(a.likelihood - b.likelihood) for a, b in zip(mixed, out["plain_f64"])),
            "max_dlogL_double_float_vs_plain": max(abs(a.likelihood - b.likelihood)
                                                   for a, b in zip(out["double_float"], out["plain_f64"]))}


SERVE_RATES = [50.0, 200.0, 300.0, 400.0, 800.0, 1400.0, 2000.0]


def serving(args):
    """Poisson arrivals over the 6 mixed-size wedges (all resident; an arrival
    picks a wedge with probability proportional to its stars), requests
    admitted against a 160 GB device-memory budget: the compensated form at
    50 to 2000 requests/s (4 lanes, batches capped at 10 ms of predicted
    device time, at most 256 requests waiting), the plain FP64 form at 1 and
    2 requests/s and the double-float form at 10, 20 and 30 requests/s
    (their throughputs on these wedges are ~3 and ~37 evaluations/s).  The
    knee is the highest rate served with p99 below 100 ms and nothing
    refused; the sustained rate the highest one completed at >= 95% of the
    arrival rate with nothing refused."""
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import native as N
    from milkywayathome_client_gb300 import serve_bench
    from milkywayathome_client_gb300 import synthetic as syn
    d = os.path.join(args.data_dir, "serving")
    m = syn.materialise(3, d)
    out = {"workload": "Poisson arrivals over 6 resident wedges (log-uniform sizes), wedge chosen by star count",
           "hbm_budget_bytes": serve_bench.HBM_BUDGET_BYTES}
    with mw.Context(0) as ctx:
        wedges = []
        for f in m["files"]:
            wid = ctx.add_wedge(mw.AstronomyParameters.read(f["params"]), mw.StarPoints.read(f["stars"]))
            wedges.append((wid, f["theta"], f["n_stars"]))
        for wid, _, _ in wedges:
            ctx.autotune(wid, N.MWSEP_MIXED_F32)
        out["resident_bytes"] = sum(ctx.wedge_bytes(w[0]) for w in wedges)
        arms = (("mixed", N.MWSEP_MIXED_F32, SERVE_RATES, 2.0, 4, 10.0, 256),
                ("plain_f64", N.MWSEP_PLAIN_F64, [1.0, 2.0], 4.0, 2, 0.0, 64),
                ("double_float", N.MWSEP_PLAIN_DF, [10.0, 20.0, 30.0], 3.0, 4, 100.0, 256))
        for name, prec, rates, secs, lanes, cap_ms, max_q in arms:
            res = serve_bench.run(rates, secs, prec, lanes, 256, d, ctx=ctx, wedges=wedges,
                                  target_batch_ms=cap_ms, max_queued=max_q)
            ok = [r["rate_req_s"] for r in res if r["p99_latency_s"] <= 0.1 and r["refused"] == 0]
            kept = [r["rate_req_s"] for r in res if r["refused"] == 0 and r["evals_per_s"] >= 0.95 * r["rate_req_s"]]
            out[name] = {"lanes": lanes, "target_batch_ms": cap_ms, "max_queued": max_q, "seconds_per_rate": secs,
                         "results": res, "knee_req_s": max(ok) if ok else None,
                         "sustained_req_s": max(kept) if kept else None,
                         "peak_evals_per_s": max(r["evals_per_s"] for r in res)}
    return out


def main():
    args = parse()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, ws, rank)
    else:
        run_gb300_arm(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
