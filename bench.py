"""Benchmark: RBF fit + evaluate throughput, mixed precision vs plain FP64, on one GB300.

Workload (default): the surface-style fit — 1M points on the ellipsoid (1, 0.7, 0.5) plus 2M
points offset by +/-0.01 along the normals (SDF values 0, +/-0.01), biharmonic3d with a degree-1
polynomial, absolute tolerance 1e-4, evaluated at 2M uniform points in the bounding box. One step
is one fit of the 3M points followed by the evaluation at the 2M query points. Inputs are seeded
synthetic data (numpy PCG64); no dataset is involved.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--scale S]

With --gpus N > 1 (torchrun, one rank per GPU) every rank fits its own replica of the workload
(replicas only: the path has no cross-GPU exchange) and value is the sum over ranks.
"""
from __future__ import annotations

import argparse
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the default sizes")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--workload", choices=["c2", "c1", "c3", "c4", "c5"], default="c2",
                    help="c2: surface fit (default, the headline); c1: 10k cube fit + 64^3 grid; "
                         "c3: 500k kriging fit + 10M queries; c4: 4096 uneven batched fits; "
                         "c5: serving stream with Poisson arrivals")
    ap.add_argument("--requests", type=int, default=600, help="c5: requests in the stream")
    ap.add_argument("--rate", type=float, default=20.0, help="c5: mean arrivals per second")
    return ap.parse_args()


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
    stats = server.stats()
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
            "timing": "host wall clock from the first arrival to the last completion"}
    print(json.dumps(line), flush=True)


def run_other(args):
    """Secondary configurations: one JSON line each, same timing rules (device time on the
    library stream, inputs resident on the device except for the batched fits, whose API takes
    host arrays)."""
    import torch

    import polatory_gb300 as pg
    from polatory_gb300 import workloads

    dev = torch.device("cuda", 0)
    stream = torch.cuda.ExternalStream(pg.stream_handle(), device=dev)
    s = args.scale
    if args.workload == "c4":
        fits = workloads.c4(n_fits=max(8, int(4096 * s)))
        model = pg.Model(pg.Triharmonic3D([1.0]), 1)
        probs = [(p, v, q) for p, v, q in fits]
        units = sum(p.shape[0] + q.shape[0] for p, v, q in fits)
        cfg = {"workload": f"{len(fits)} uneven fits, N log-uniform 200..20000 (sum {units}), "
                           "triharmonic3d degree 1, tol 1e-5, 4096 queries each",
               "n_fits": len(fits)}
        prec = pg.MIXED

        def step():
            return pg.fit_batch(model, probs, 1e-5, precision=prec, return_weights=False)
    else:
        if args.workload == "c1":
            pts, vals, q = workloads.c1()
            model = pg.Model(pg.Biharmonic3D([1.0]), 1)
            tol = 1e-5
            cfg = {"workload": "10000 uniform points, biharmonic3d degree 1, tol 1e-5, 64^3 grid"}
        else:
            n = max(10000, int(500_000 * s))
            pts, vals, q, aniso = workloads.c3(n=n, n_eval=max(10000, int(10_000_000 * s)))
            rbf = pg.CovExponential([1.0, 0.2])
            rbf.anisotropy = aniso  # diag(1, 1, 2): range scale 1:1:0.5
            model = pg.Model(rbf, 0)
            model.nugget = 1e-3
            tol = 1e-4
            cfg = {"workload": f"{n} GMM points, cov_exponential range 0.2 aniso 1:1:0.5, nugget "
                               f"1e-3, degree 0, tol 1e-4, {q.shape[0]} uniform queries"}
        units = pts.shape[0] + q.shape[0]
        pts_d = torch.from_numpy(pts).to(dev)
        vals_d = torch.from_numpy(vals).to(dev)
        q_d = torch.from_numpy(q).to(dev)
        out_d = torch.empty(q.shape[0], dtype=torch.float64, device=dev)
        interp = pg.Interpolant(model, pg.MIXED)

        def step():
            interp.fit_device(pts_d, vals_d, tol)
            interp.evaluate_device(q_d, out_d)
            return interp.fit_stats
    for _ in range(args.warmup):
        step()
    pg.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        info = step()
    ev1.record(stream)
    pg.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms = ev0.elapsed_time(ev1) if args.workload != "c4" else wall * 1e3
    line = {"metric": f"{args.workload} fit+eval points/s (mixed precision)", "value": units * args.steps / (ms * 1e-3),
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "data": "synthetic",
            "config": cfg}
    if args.workload == "c4":
        its = [r["iterations"] for r in info]
        line["fit"] = {"iterations_mean": float(np.mean(its)), "iterations_max": int(max(its)),
                       "failed": int(sum(r["status"] != 0 for r in info)),
                       "timing": "host wall clock (batched API takes host arrays)"}
    else:
        line["fit"] = info
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


def workload(scale: float):
    from polatory_gb300 import workloads

    ns = max(1000, int(1_000_000 * scale))
    pts, vals, q = workloads.c2(n_surface=ns, n_eval=max(1000, int(2_000_000 * scale)))
    cfg = {
        "workload": f"surface SDF fit: {pts.shape[0]} points (ellipsoid 1/0.7/0.5, +/-0.01 "
                    f"offsets), biharmonic3d degree 1, tol 1e-4, {q.shape[0]} uniform queries",
        "n_fit": int(pts.shape[0]), "n_eval": int(q.shape[0]), "rbf": "bh3 (-r)",
        "poly_degree": 1, "tolerance": 1e-4, "precision": "mixed (FP32 near/far field, "
        "FP64 Krylov + residual)",
        "l2_policy": "inputs and working set larger than L2 (no flush needed)",
    }
    return pts, vals, q, cfg


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


def cpu_baseline(pts, vals, q, budget_n_fit=3000, n_eval=2000):
    """The oracle (FP64 C restatement: exact dense fit + direct sums) on the host cores, on a
    bounded subsample of the same workload."""
    import oracle
    import polatory_gb300 as pg

    g = np.random.Generator(np.random.PCG64(77))
    idx = np.sort(g.choice(pts.shape[0], size=min(budget_n_fit, pts.shape[0]), replace=False))
    sp, sv = pts[idx], vals[idx]
    sq = q[g.choice(q.shape[0], size=min(n_eval, q.shape[0]), replace=False)]
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    t0 = time.perf_counter()
    w = oracle.fit_exact(model, sp, sv)
    oracle.direct_evaluate(model, sp, w, sq)
    dt = time.perf_counter() - t0
    return {"value": (sp.shape[0] + sq.shape[0]) / dt, "unit": UNIT, "cores": oracle.num_threads(),
            "kind": "port",
            "sample": f"exact dense FP64 fit of {sp.shape[0]} sampled data points + direct "
                      f"evaluation at {sq.shape[0]} sampled queries ({dt:.2f} s)"}


def exact_residual_sample(pg, model, pts, vals, w, n_sample=10000, seed=11):
    """The mixed fit's residual recomputed with exact FP64 direct sums at n_sample data points
    drawn at random (outside the timed region): max |value - (sum_j w_j phi + polynomial)|."""
    g = np.random.Generator(np.random.PCG64(seed))
    idx = np.sort(g.choice(pts.shape[0], min(n_sample, pts.shape[0]), replace=False))
    n = pts.shape[0]
    lo, hi = pts.min(0), pts.max(0)
    ev = pg.FmmEvaluator(model.rbfs[0], np.concatenate([lo, hi]), precision=pg.PLAIN)
    ev.configure(backend=1)
    ev.set_source_points(pts)
    ev.set_target_points(pts[idx])
    ev.set_weights(w[:n])
    fit = ev.evaluate()
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
    """The reference arm: the reference's CPU path as restated by the oracle (the reference
    itself cannot be built here), timed on the host cores on a bounded sample per step."""
    rank, world, local, dist = dist_setup(args)
    if rank != 0:
        return
    pts, vals, q, cfg = workload(args.scale)
    for _ in range(args.warmup):
        cpu_baseline(pts, vals, q, budget_n_fit=1000, n_eval=500)
    vals_s = []
    base = None
    for _ in range(args.steps):
        base = cpu_baseline(pts, vals, q)
        vals_s.append(base["value"])
    v = float(np.mean(vals_s))
    base["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": cfg, "cpu_baseline": base,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference not buildable here (Eigen/ScalFMM3 absent); oracle FP64 port timed"}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "c5":
        run_serving(args)
        return
    if args.workload != "c2":
        run_other(args)
        return
    import torch

    rank, world, local, dist = dist_setup(args)
    import polatory_gb300 as pg

    pg._lib.check(pg._lib.lib.pgpu_set_device(local))
    torch.cuda.set_device(local)
    pts, vals, q, cfg = workload(args.scale)
    n_units = pts.shape[0] + q.shape[0]
    dev = torch.device("cuda", local)
    pts_d = torch.from_numpy(pts).to(dev)
    vals_d = torch.from_numpy(vals).to(dev)
    q_d = torch.from_numpy(q).to(dev)
    out_d = torch.empty(q.shape[0], dtype=torch.float64, device=dev)
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    stream = torch.cuda.ExternalStream(pg.stream_handle(), device=dev)

    def step(interp):
        interp.fit_device(pts_d, vals_d, 1e-4)
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
    exact_res = exact_residual_sample(pg, model, pts, vals, interp.weights) if rank == 0 else None

    # End to end through the C ABI with host buffers (copies inside the timed region).
    e2e_interp = pg.Interpolant(model, pg.MIXED)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(max(1, min(args.steps, 2))):
        e2e_interp.fit(pts, vals, 1e-4)
        host_out = e2e_interp.evaluate(q)
    e2e_s = (time.perf_counter() - t0) / max(1, min(args.steps, 2))
    e2e = {"value": world * n_units / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(pts.nbytes + vals.nbytes + q.nbytes),
           "d2h_bytes_per_step": int(host_out.nbytes)}

    plain = None
    if not args.no_plain:
        pi = pg.Interpolant(model, pg.PLAIN)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step(pi)
        pg.synchronize()
        dt = time.perf_counter() - t0
        plain_out = out_d.cpu().numpy()
        err = float(np.max(np.abs(mixed_out - plain_out)))
        plain = {"value": n_units / dt, "unit": UNIT, "seconds": dt,
                 "iterations": pi.fit_stats["iterations"],
                 "mixed_vs_plain_max_abs_err": err, "speedup_mixed_over_plain": value / world / (n_units / dt)}

    if rank != 0:
        return
    # Roofline of the dominant kernel (device time per region from the live CUDA events).
    dom_name, dom = max(report.items(), key=lambda kv: kv[1]["ms"])
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    roof = roofline(dom_name, dom, ms, sms)
    top = sorted(report.items(), key=lambda kv: -kv[1]["ms"])[:6]
    regions = {k: {kk: vv for kk, vv in roofline(k, v, ms, sms).items() if kk != "kernel"}
               for k, v in top}
    cpu = None if args.no_cpu else cpu_baseline(pts, vals, q)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
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


if __name__ == "__main__":
    main()
