"""Benchmark: RBF fit + evaluate throughput, mixed precision vs plain FP64, on one GB300.

Workloads (seeded synthetic data, numpy PCG64; no dataset is involved):
  c2 (default, the headline): 1M points on the ellipsoid (1, 0.7, 0.5) plus 2M points offset by
     +/-0.01 along the normals (SDF values 0, +/-0.01), biharmonic3d with a degree-1 polynomial,
     absolute tolerance 1e-4, evaluated at 2M uniform points in the bounding box;
  c1: 10,000 uniform points, biharmonic3d degree 1, tol 1e-5, evaluated on a 64^3 grid;
  c3: 500k Gaussian-mixture points, cov_exponential (range 0.2, anisotropy 1:1:0.5, nugget 1e-3),
     degree 0, tol 1e-4, 10M uniform queries;
  c4: 4,096 uneven triharmonic fits (batched API); c5: a serving stream.
One step of c1/c2/c3 is one fit of the data points followed by the evaluation at the queries.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload c2]
                  [--scale S]

With --gpus N > 1 (torchrun, one rank per GPU) every rank fits its own replica of the workload
(replicas only: the path has no cross-GPU exchange) and value is the sum over ranks.

--impl reference times the CPU stand-in for the reference (the reference itself, C++ with Eigen
and ScalFMM3, cannot be built here): the oracle's exact dense FP64 solve plus exact direct
evaluation, on the host cores. It never loads the product library. c1 runs whole on both arms;
c2 and c3 run a bounded sample per step (12,000 data points, 200,000 queries) whose rate does not
carry over to the whole configuration (a dense solve scales as n^3), and c4 a sample of its fits.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "fit+eval points/s (mixed precision, 1e-4 abs err vs plain FP64)"
UNIT = "points/s"
# Largest fit the dense CPU stand-in runs in full (an n^2 FP64 matrix, 2/3 n^3 flops).
DENSE_LIMIT = 12_000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the default sizes (c2, c3, c4)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--workload", choices=["c2", "c1", "c3", "c4", "c5"], default="c2",
                    help="c2: surface fit (default, the headline); c1: 10k cube fit + 64^3 grid; "
                         "c3: 500k kriging fit + 10M queries; c4: 4096 uneven batched fits; "
                         "c5: serving stream with Poisson arrivals")
    ap.add_argument("--requests", type=int, default=600, help="c5: requests in the stream")
    ap.add_argument("--rate", type=float, default=20.0, help="c5: mean arrivals per second")
    return ap.parse_args()


def load_workloads():
    """The numpy-only input generator, loaded by path so that the reference arm never imports
    the product package (whose import loads the CUDA library)."""
    spec = importlib.util.spec_from_file_location("_pgpu_workloads",
                                                  ROOT / "polatory_gb300" / "workloads.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def make_workload(name: str, scale: float) -> dict:
    """Inputs, model description, tolerance and config of one single-fit workload."""
    W = load_workloads()
    if name == "c1":
        pts, vals, q = W.c1()
        md = {"kind": "bh3", "params": [1.0], "poly_degree": 1, "nugget": 0.0, "aniso": None}
        tol = 1e-5
        desc = (f"uniform cube fit: {pts.shape[0]} points, biharmonic3d degree 1, tol 1e-5, "
                f"64^3 grid ({q.shape[0]} queries)")
    elif name == "c2":
        ns = max(1000, int(1_000_000 * scale))
        pts, vals, q = W.c2(n_surface=ns, n_eval=max(1000, int(2_000_000 * scale)))
        md = {"kind": "bh3", "params": [1.0], "poly_degree": 1, "nugget": 0.0, "aniso": None}
        tol = 1e-4
        desc = (f"surface SDF fit: {pts.shape[0]} points (ellipsoid 1/0.7/0.5, +/-0.01 offsets), "
                f"biharmonic3d degree 1, tol 1e-4, {q.shape[0]} uniform queries")
    elif name == "c3":
        n = max(10_000, int(500_000 * scale))
        pts, vals, q, aniso = W.c3(n=n, n_eval=max(10_000, int(10_000_000 * scale)))
        md = {"kind": "exp", "params": [1.0, 0.2], "poly_degree": 0, "nugget": 1e-3, "aniso": aniso}
        tol = 1e-4
        desc = (f"kriging fit: {n} Gaussian-mixture points, cov_exponential psill 1 range 0.2 "
                f"anisotropy 1:1:0.5, nugget 1e-3, degree 0, tol 1e-4, {q.shape[0]} uniform queries")
    else:
        raise ValueError(name)
    cfg = {"workload": desc, "n_fit": int(pts.shape[0]), "n_eval": int(q.shape[0]),
           "rbf": {"bh3": "bh3 (-r)", "exp": "cov_exponential"}[md["kind"]],
           "poly_degree": md["poly_degree"], "tolerance": tol,
           "precision": "mixed (FP32 near/far field, FP64 Krylov + residual)",
           "l2_policy": "inputs and working set larger than L2 (no flush needed)"
           if pts.shape[0] + q.shape[0] > 1_000_000 else
           "inputs smaller than L2; every step refits and rebuilds its trees (no flush)"}
    return {"name": name, "pts": pts, "vals": vals, "q": q, "model": md, "tol": tol, "cfg": cfg}


def pg_model(pg, md):
    rbf = pg.Biharmonic3D(md["params"]) if md["kind"] == "bh3" else pg.CovExponential(md["params"])
    if md["aniso"] is not None:
        rbf.anisotropy = md["aniso"]
    model = pg.Model(rbf, md["poly_degree"])
    model.nugget = md["nugget"]
    return model


def oracle_model(md):
    import oracle

    return oracle.model(md["kind"], md["params"], md["poly_degree"], md["nugget"], md["aniso"])


def run_serving(args):
    """Serving stream: Poisson arrivals, 70% evaluations (1k-1M query points, log-uniform)
    against resident models and 30% fits (N log-uniform 1k-200k, biharmonic3d or cov_exponential
    with range 0.1-0.5, tol 1e-4), admitted against a 150 GB device-memory budget. Inputs are
    host arrays (the serving API copies them in); latency is submit-to-completion on the host
    clock. Eight resident models are fitted before the timed stream."""
    import polatory_gb300 as pg

    g = np.random.Generator(np.random.PCG64(5))
    n_req = max(20, int(args.requests))
    qpool = g.random((1_000_000, 3))
    fpool = g.random((200_000, 3))
    fvals = np.sin(2 * np.pi * fpool[:, 0]) * np.cos(2 * np.pi * fpool[:, 1]) + fpool[:, 2] ** 2

    def model_for(rng):
        if rng.random() < 0.5:
            return pg.Model(pg.Biharmonic3D([1.0]), 1)
        return pg.Model(pg.CovExponential([1.0, float(rng.uniform(0.1, 0.5))]), 0)

    def log_uniform(rng, lo, hi):
        return int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))

    n_slots = 8
    server = pg.Server(n_workers=8, hbm_budget_bytes=150 * 10**9)
    for k in range(n_slots):
        n = log_uniform(g, 1000, 200_000)
        t = server.submit_fit(k, model_for(g), fpool[:n], fvals[:n], 1e-4, precision=pg.MIXED)
        st = server.wait(t)
        assert st[0] == 0, st[3]
    plan = []
    t_arr = 0.0
    for i in range(n_req):
        t_arr += g.exponential(1.0 / args.rate)
        if g.random() < 0.7:
            plan.append((t_arr, "evaluate", int(g.integers(n_slots)), log_uniform(g, 1000, 1_000_000)))
        else:
            plan.append((t_arr, "fit", int(g.integers(n_slots)), log_uniform(g, 1000, 200_000)))
    models = [model_for(g) for _ in range(n_req)]
    tickets = []
    # Device memory in use (the whole device, from cudaMemGetInfo) sampled through the stream.
    import torch

    mem = {"max": 0}
    mem_stop = threading.Event()

    def sample_memory():
        while not mem_stop.wait(0.5):
            free, total = torch.cuda.mem_get_info()
            mem["max"] = max(mem["max"], total - free)

    sampler = threading.Thread(target=sample_memory, daemon=True)
    sampler.start()
    start = time.perf_counter()
    for (ta, kind, slot, n), m in zip(plan, models):
        delay = start + ta - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        if kind == "evaluate":
            t = server.submit_evaluate(slot, qpool[:n], precision=pg.MIXED)
        else:
            t = server.submit_fit(slot, m, fpool[:n], fvals[:n], 1e-4, precision=pg.MIXED)
        tickets.append((t, kind, n))
    lat = {"fit": [], "evaluate": []}
    failed = 0
    errors = []
    points = 0
    for t, kind, n in tickets:
        st, latency, _, msg = server.wait(t)
        if st != 0:
            failed += 1
            if len(errors) < 3:
                errors.append(f"{kind} n={n}: status {st}: {msg}")
            continue
        lat[kind].append(latency)
        points += n
    wall = time.perf_counter() - start
    mem_stop.set()
    sampler.join()
    stats = server.stats()
    cache = pg.operator_cache_stats()
    server.close()
    allv = lat["fit"] + lat["evaluate"]

    def pct(v, q):
        return float(np.percentile(v, q)) if v else None

    line = {"metric": "c5 serving points/s (mixed precision)", "value": points / wall,
            "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": wall * 1e3,
            "higher_is_better": True, "data": "synthetic",
            "config": {"workload": f"{n_req} requests, Poisson arrivals at {args.rate}/s, 70% "
                                   "evaluate 1k-1M queries on 8 resident models, 30% fit 1k-200k "
                                   "(bh3 degree 1 or cov_exponential range 0.1-0.5), tol 1e-4, "
                                   "150 GB budget, 8 workers"},
            "latency_s": {"p50": pct(allv, 50), "p99": pct(allv, 99),
                          "fit_p50": pct(lat["fit"], 50), "fit_p99": pct(lat["fit"], 99),
                          "evaluate_p50": pct(lat["evaluate"], 50),
                          "evaluate_p99": pct(lat["evaluate"], 99)},
            "failed": failed, "errors": errors, "peak_bytes": stats["peak_bytes"],
            "device_used_max_bytes": mem["max"], "operator_cache": cache,
            "timing": "host wall clock from the first arrival to the last completion"}
    print(json.dumps(line), flush=True)


def run_batched(args):
    """Batched uneven fits (c4): one JSON line. The batched API takes host arrays, so the step
    is timed on the host clock around the whole batch (copies included)."""
    import polatory_gb300 as pg

    W = load_workloads()
    fits = W.c4(n_fits=max(8, int(4096 * args.scale)))
    model = pg.Model(pg.Triharmonic3D([1.0]), 1)
    probs = [(p, v, q) for p, v, q in fits]
    units = sum(p.shape[0] + q.shape[0] for p, v, q in fits)
    cfg = {"workload": f"{len(fits)} uneven fits, N log-uniform 200..20000 (sum {units}), "
                       "triharmonic3d degree 1, tol 1e-5, 4096 queries each",
           "n_fits": len(fits)}

    def step():
        return pg.fit_batch(model, probs, 1e-5, precision=pg.MIXED, return_weights=False)

    for _ in range(args.warmup):
        step()
    pg.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        info = step()
    pg.synchronize()
    ms = (time.perf_counter() - t0) * 1e3
    its = [r["iterations"] for r in info]
    line = {"metric": "c4 fit+eval points/s (mixed precision)", "value": units * args.steps / (ms * 1e-3),
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "data": "synthetic",
            "config": cfg,
            "fit": {"iterations_mean": float(np.mean(its)), "iterations_max": int(max(its)),
                    "failed": int(sum(r["status"] != 0 for r in info)),
                    "timing": "host wall clock (batched API takes host arrays)"}}
    print(json.dumps(line), flush=True)


def roofline(name, region, ms_step, sms):
    """Achieved rate of one profiled region against the peak of the unit that bounds it.

    Flop regions count algorithmic flops (pairs x flops per pair, 2 p^6 per M2L interaction);
    the tensor-core M2L executes three TF32 products per algorithmic product (head/tail split),
    and is compared with the TF32 dense rate, half the measured BF16 rate. Byte regions count
    algorithmic bytes. traffic: DRAM bytes per launch from an ncu capture of the same kernel
    (profiles/traffic.json), or null."""
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    clk_max = peaks.get("sm_max_mhz", 2070.0)
    fp32_peak = sms * 128 * 2 * clk_max * 1e6 / 1e12
    fp64_peak = sms * 2 * 2 * clk_max * 1e6 / 1e12
    secs = region["ms"] * 1e-3
    if region["bytes"] > 0 and region["flops"] / max(region["bytes"], 1) < 4:
        roof = {"bound": "hbm", "achieved": region["bytes"] / secs / 1e9,
                "peak": peaks.get("hbm_gbs", 6800.0), "unit": "GB/s",
                "peak_source": "hbm_gbs of measured" if "hbm_gbs" in peaks else "fallback 6.8 TB/s"}
    elif name == "fmm_m2l_tc":
        bf16 = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops", 1900.0))
        roof = {"bound": "tensor", "achieved": 3.0 * region["flops"] / secs / 1e12,
                "peak": bf16 / 2.0, "unit": "TFLOP/s",
                "peak_source": "TF32 dense = half the sustained BF16 rate of measured",
                "useful_tflops": region["flops"] / secs / 1e12}
    else:
        f64 = "f64" in name
        roof = {"bound": "fp64-cuda-core" if f64 else "fp32-cuda-core",
                "achieved": region["flops"] / secs / 1e12,
                "peak": fp64_peak if f64 else fp32_peak, "unit": "TFLOP/s",
                "peak_source": f"nominal {'FP64' if f64 else 'FP32'} CUDA-core FMA rate: {sms} SMs x "
                               f"{2 if f64 else 128} x 2 flops x {clk_max:.0f} MHz"}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["kernel"] = name
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        t = json.loads(tf.read_text()).get(name)
        if t:
            traffic = t["dram_bytes_per_launch"]
    roof["traffic"] = traffic
    roof["launches"] = region["calls"]
    roof["ms_total"] = region["ms"]
    roof["share_of_step"] = region["ms"] / ms_step
    return roof


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device),
                                      f"--query-gpu={self.Q}", "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, name in enumerate(names):
                if len(s) > 5 + k and s[5 + k].strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def oracle_time(wl, n_fit=None, n_eval=None, seed=77):
    """Times the oracle (FP64 C restatement, all host threads): an exact dense solve of the fit
    system and exact direct evaluation at the queries. n_fit/n_eval None: the whole workload;
    otherwise a seeded random subsample of that many data points and queries."""
    import oracle

    pts, vals, q = wl["pts"], wl["vals"], wl["q"]
    if n_fit is not None:
        g = np.random.Generator(np.random.PCG64(seed))
        idx = np.sort(g.choice(pts.shape[0], size=min(n_fit, pts.shape[0]), replace=False))
        pts, vals = pts[idx], vals[idx]
        q = q[g.choice(q.shape[0], size=min(n_eval, q.shape[0]), replace=False)]
    m = oracle_model(wl["model"])
    t0 = time.perf_counter()
    w = oracle.fit_exact(m, pts, vals)
    t1 = time.perf_counter()
    out = oracle.direct_evaluate(m, pts, w, q)
    t2 = time.perf_counter()
    return {"seconds": t2 - t0, "fit_s": t1 - t0, "eval_s": t2 - t1, "n_fit": int(pts.shape[0]),
            "n_eval": int(q.shape[0]), "threads": oracle.num_threads(), "weights": w, "out": out}


def cpu_baseline(wl):
    """The reported CPU baseline (never a target). Configurations within DENSE_LIMIT run in full;
    larger ones run a bounded subsample, whose rate does not carry over to the configuration
    (a dense solve costs n^3), and say so."""
    n = wl["pts"].shape[0]
    if n <= DENSE_LIMIT:
        r = oracle_time(wl)
        return {"value": (r["n_fit"] + r["n_eval"]) / r["seconds"], "unit": UNIT,
                "cores": r["threads"], "kind": "port", "comparable": True,
                "sample": f"the whole configuration: exact dense FP64 fit of {r['n_fit']} points "
                          f"({r['fit_s']:.2f} s) + direct evaluation at {r['n_eval']} queries "
                          f"({r['eval_s']:.2f} s)"}
    r = oracle_time(wl, n_fit=3000, n_eval=2000)
    full_s = r["fit_s"] * (n / r["n_fit"]) ** 3
    return {"value": (r["n_fit"] + r["n_eval"]) / r["seconds"], "unit": UNIT, "cores": r["threads"],
            "kind": "port", "comparable": False,
            "sample": f"exact dense FP64 fit of {r['n_fit']} sampled data points + direct evaluation "
                      f"at {r['n_eval']} sampled queries ({r['seconds']:.2f} s); a dense solve scales "
                      f"as n^3, so this rate does not carry over to the {n}-point fit (the same solve "
                      f"would take ~{full_s:.2e} s there)"}


def exact_residual_sample(pg, model, wl, w, n_sample=10000, seed=11):
    """The fit's residual recomputed with exact FP64 direct sums (the library's direct backend,
    itself checked against the oracle) at n_sample data points drawn at random, outside the
    timed region: max |value - (sum_j w_j phi + nugget w_i + polynomial)|."""
    pts, vals = wl["pts"], wl["vals"]
    g = np.random.Generator(np.random.PCG64(seed))
    idx = np.sort(g.choice(pts.shape[0], min(n_sample, pts.shape[0]), replace=False))
    n = pts.shape[0]
    lo, hi = pts.min(0), pts.max(0)
    ev = pg.FmmEvaluator(model.rbfs[0], np.concatenate([lo, hi]), precision=pg.PLAIN)
    ev.configure(backend=1)
    ev.set_source_points(pts)
    ev.set_target_points(pts[idx])
    ev.set_weights(w[:n])
    fit = ev.evaluate() + model.nugget * w[:n][idx]
    c = w[n:]
    q = pts[idx]
    if c.shape[0] >= 1:
        fit = fit + c[0]
    if c.shape[0] >= 4:
        fit = fit + c[1] * q[:, 0] + c[2] * q[:, 1] + c[3] * q[:, 2]
    return {"points": int(idx.shape[0]), "max_abs": float(np.max(np.abs(fit - vals[idx])))}


def combine_ranks(dist, ms, world, n_units, steps, device):
    """Replicas: every rank ran the same workload; the job's time is the slowest rank's
    (max over ranks, after a barrier) and its value the units of all ranks over that time."""
    import torch

    t_max = ms
    if dist is not None:
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
        dist.barrier()
    return t_max, world * n_units * steps / (t_max * 1e-3)


def dist_setup(args):
    if args.gpus <= 1 or "RANK" not in os.environ:
        return 0, 1, 0, None
    import torch.distributed as dist

    rank = int(os.environ["RANK"])
    world = int(os.environ["WORLD_SIZE"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    import torch

    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return rank, world, local, dist


def run_reference(args):
    """The reference arm: the CPU stand-in for the reference (the oracle's exact dense FP64 solve
    and direct sums; the reference itself cannot be built here) on the host cores, for the same
    configuration. A configuration whose dense system fits (c1) runs whole; larger ones (c2, c3)
    run a bounded sample of it per step (12,000 of its data points and 200,000 of its queries),
    and c4 a sample of its fits; the line says so. Rank 0 alone runs it; the product library is
    never loaded."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    base = {"impl": "reference", "metric": METRIC, "unit": UNIT, "n_gpus": args.gpus,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic"}
    note = ("the reference cannot be built here (Eigen/Boost/ScalFMM3 absent, no network); the "
            "oracle's exact dense FP64 solve and direct sums stand in for its FMM/FGMRES/RAS path")
    if args.workload == "c5":
        print(json.dumps({**base, "unavailable":
                          "c5: the reference (C++ with Eigen/Boost/ScalFMM3) cannot be built here, "
                          "and a serving stream of fits of up to 200,000 points has no bounded "
                          "sample for a dense solve that keeps its latency distribution"}), flush=True)
        return
    # Each step is seconds to tens of seconds: the step counts are capped so that the run ends
    # within a few minutes, and the counts run are reported.
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, 3))
    if args.workload == "c4":
        W = load_workloads()
        fits = W.c4(n_fits=max(8, int(4096 * args.scale)))
        # The batch's first fits of at most DENSE_LIMIT points, up to 16 of them.
        sample = [f for f in fits if f[0].shape[0] <= DENSE_LIMIT][:16]
        md = {"kind": "th3", "params": [1.0], "poly_degree": 1, "nugget": 0.0, "aniso": None}

        def one_step():
            t = 0.0
            for p, v, q in sample:
                r = oracle_time({"pts": p, "vals": v, "q": q, "model": md})
                t += r["seconds"]
            return t

        for _ in range(warm):
            one_step()
        secs = [one_step() for _ in range(steps)]
        units = sum(p.shape[0] + q.shape[0] for p, v, q in sample)
        v = units * steps / sum(secs)
        import oracle

        line = {**base, "metric": "c4 fit+eval points/s (mixed precision)", "value": v,
                "steps": steps, "warmup": warm, "ms_per_step": 1e3 * sum(secs) / steps,
                "config": {"workload": f"{len(fits)} uneven fits, N log-uniform 200..20000, "
                                       "triharmonic3d degree 1, tol 1e-5, 4096 queries each",
                           "n_fits": len(fits)},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                                 "comparable": False,
                                 "sample": f"per step the batch's first {len(sample)} fits of at most "
                                           f"{DENSE_LIMIT} points ({units} points with their queries), "
                                           "each an exact dense FP64 fit + direct evaluation"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "requested": {"steps": args.steps, "warmup": args.warmup}, "note": note}
        print(json.dumps(line), flush=True)
        return
    wl = make_workload(args.workload, args.scale)
    n = wl["pts"].shape[0]
    whole = n <= DENSE_LIMIT
    n_fit = None if whole else DENSE_LIMIT
    n_eval = None if whole else min(wl["q"].shape[0], 200_000)
    for _ in range(warm):
        oracle_time(wl, n_fit, n_eval)
    secs = []
    r = None
    for k in range(steps):
        r = oracle_time(wl, n_fit, n_eval, seed=77 + k)
        secs.append(r["seconds"])
    units = r["n_fit"] + r["n_eval"]
    v = units * steps / sum(secs)
    if whole:
        sample = (f"the whole configuration per step: exact dense FP64 fit of {r['n_fit']} points "
                  f"({r['fit_s']:.2f} s) + direct evaluation at {r['n_eval']} queries "
                  f"({r['eval_s']:.2f} s)")
    else:
        full_s = r["fit_s"] * (n / r["n_fit"]) ** 3
        sample = (f"a bounded sample per step: exact dense FP64 fit of {r['n_fit']} of the {n} data "
                  f"points ({r['fit_s']:.2f} s) + direct evaluation at {r['n_eval']} of the "
                  f"{wl['q'].shape[0]} queries ({r['eval_s']:.2f} s); a dense solve scales as n^3 "
                  f"where the reference's FMM/FGMRES/RAS path scales near n log n, so this rate "
                  f"does not carry over to the whole configuration (the dense solve of all {n} "
                  f"points would take ~{full_s:.2e} s)")
    line = {**base, "value": v, "steps": steps, "warmup": warm, "ms_per_step": 1e3 * sum(secs) / steps,
            "config": wl["cfg"],
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": r["threads"], "kind": "port",
                             "comparable": whole, "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "requested": {"steps": args.steps, "warmup": args.warmup}, "note": note}
    print(json.dumps(line), flush=True)


def run_fit_eval(args):
    """Our arm on a single-fit workload (c1, c2, c3): W warm-up and K timed steps on the device
    (CUDA events on the library stream), then the end-to-end run with host buffers, the plain
    FP64 comparison (one warm-up step, one timed step) and the CPU baseline."""
    import torch

    rank, world, local, dist = dist_setup(args)
    import polatory_gb300 as pg

    pg._lib.check(pg._lib.lib.pgpu_set_device(local))
    torch.cuda.set_device(local)
    wl = make_workload(args.workload, args.scale)
    pts, vals, q, tol, cfg = wl["pts"], wl["vals"], wl["q"], wl["tol"], wl["cfg"]
    n_units = pts.shape[0] + q.shape[0]
    dev = torch.device("cuda", local)
    pts_d = torch.from_numpy(pts).to(dev)
    vals_d = torch.from_numpy(vals).to(dev)
    q_d = torch.from_numpy(q).to(dev)
    out_d = torch.empty(q.shape[0], dtype=torch.float64, device=dev)
    model = pg_model(pg, wl["model"])
    stream = torch.cuda.ExternalStream(pg.stream_handle(), device=dev)

    def step(interp):
        interp.fit_device(pts_d, vals_d, tol)
        interp.evaluate_device(q_d, out_d)

    interp = pg.Interpolant(model, pg.MIXED)
    for _ in range(args.warmup):
        step(interp)
    pg.synchronize()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    pg.profile_reset()
    pg.profile_enable(True)
    launches0 = pg.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    iters = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step(interp)
            iters.append(interp.fit_stats["iterations"])
        ev1.record(stream)
        pg.synchronize()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = pg.launch_count() - launches0
    report = pg.profile_report()
    pg.profile_enable(False)
    t_max, value = combine_ranks(dist, ms, world, n_units, args.steps, dev)
    mixed_out = out_d.cpu().numpy()
    stats = interp.fit_stats
    exact_res = exact_residual_sample(pg, model, wl, interp.weights) if rank == 0 else None

    # End to end through the C ABI with host buffers (copies inside the timed region).
    e2e_interp = pg.Interpolant(model, pg.MIXED)
    torch.cuda.synchronize()
    n_e2e = max(1, min(args.steps, 2))
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        e2e_interp.fit(pts, vals, tol)
        host_out = e2e_interp.evaluate(q)
    e2e_s = (time.perf_counter() - t0) / n_e2e
    e2e = {"value": world * n_units / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(pts.nbytes + vals.nbytes + q.nbytes),
           "d2h_bytes_per_step": int(host_out.nbytes), "timing": "host wall clock, host buffers"}

    plain = None
    if not args.no_plain:
        pi = pg.Interpolant(model, pg.PLAIN)
        step(pi)  # warm-up: builds the FP64 far-field operator tables
        pg.synchronize()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        step(pi)
        p1.record(stream)
        pg.synchronize()
        torch.cuda.synchronize()
        dt = p0.elapsed_time(p1) * 1e-3
        plain_out = out_d.cpu().numpy()
        err = float(np.max(np.abs(mixed_out - plain_out)))
        # The same comparison with both interpolants evaluated at accuracy 1e-6 (the estimator's
        # far-field order, or exact sums) at 100,000 of the queries: the difference of the two
        # fits without the default order-6 evaluation error of either.
        sub = q[np.random.Generator(np.random.PCG64(12)).choice(q.shape[0], min(100_000, q.shape[0]),
                                                               replace=False)]
        err_acc = float(np.max(np.abs(interp.evaluate(sub, accuracy=1e-6) -
                                      pi.evaluate(sub, accuracy=1e-6))))
        plain = {"value": n_units / dt, "unit": UNIT, "seconds": dt, "warmup": 1, "steps": 1,
                 "iterations": pi.fit_stats["iterations"], "residual": pi.fit_stats["residual"],
                 "mixed_vs_plain_max_abs_err": err, "error_bound": 1e-4,
                 "mixed_vs_plain_max_abs_err_at_accuracy_1e-6": err_acc,
                 "speedup_mixed_over_plain": value / world / (n_units / dt),
                 "timing": "CUDA events on the library stream after one warm-up step"}

    if rank != 0:
        return
    # Roofline of the dominant kernel (device time per region from the live CUDA events).
    dom_name, dom = max(report.items(), key=lambda kv: kv[1]["ms"])
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    roof = roofline(dom_name, dom, ms, sms)
    top = sorted(report.items(), key=lambda kv: -kv[1]["ms"])[:8]
    regions = {k: {kk: vv for kk, vv in roofline(k, v, ms, sms).items() if kk != "kernel"}
               for k, v in top}
    cpu = None if args.no_cpu else cpu_baseline(wl)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": cfg, "e2e": e2e, "gpu_launches": int(launches), "roofline": roof,
        "regions": regions,
        "cpu_baseline": cpu, "clocks": clk.summary(), "plain_fp64": plain,
        "fit": {"iterations": iters, "levels": stats["levels"], "residual": stats["residual"],
                "fp64_residual_sample": exact_res,
                "setup_s": stats["setup_seconds"], "solve_s": stats["solve_seconds"],
                "n_domains": stats["n_domains"]},
        "profile_ms": {k: round(v["ms"], 3) for k, v in sorted(report.items(), key=lambda kv: -kv[1]["ms"])},
        "profile_rate": {k: {"calls": v["calls"],
                             "tflops": round(v["flops"] / (v["ms"] * 1e-3) / 1e12, 3) if v["ms"] > 0 else None,
                             "gbs": round(v["bytes"] / (v["ms"] * 1e-3) / 1e9, 1) if v["ms"] > 0 else None}
                         for k, v in report.items()},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c5":
        run_serving(args)
    elif args.workload == "c4":
        run_batched(args)
    else:
        run_fit_eval(args)


if __name__ == "__main__":
    main()
