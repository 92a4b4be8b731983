"""Benchmark of feyntrop's tropical sampling + integrand evaluation loop on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one step): one integration of the planar double box (6 vertices,
7 edges, Minkowski kinematics with the contour deformation, lambda = 0.5, 2 eps
orders) with N = 1e8 samples of the seed's xoshiro256+ stream, in mixed precision
(FP32 integrand, FP64 sector decisions and FP64 re-evaluation of flagged samples).
The plain-FP64 GPU form of the same step is timed beside it.  Inputs are synthetic
(seeded kinematics); nothing is read from disk.

Timing: W untimed steps, then K steps, each bracketed by CUDA events on the stream
the kernels run on; the L2 cache is flushed (256 MiB write) between steps, outside
the events.  A barrier and a device synchronize bracket the timed loop; the
reported time is the max over ranks.  `e2e` repeats the step through the public
API as a user calls it (plan creation with host preprocessing and the upload of
the table, integration, result read-back) timed on the host.

Batched form (`batched` in the line, --batched both|scan|mixed|none): a whole seeded
batch of integrals per run, one CUDA graph launch with one persistent sampling launch
per topology class, mixed precision against plain FP64 on the same integrals.  By
default both workloads: the 4096-point box-pentagon kinematic scan and the mixed
uneven batch (1536 integrals of four topologies), each with the per-sample error of
every kernel class.

Multi-GPU (torchrun): rank r integrates its own block of N samples of the same
stream (samples [rN, (r+1)N)); the merged moments equal a single run over all
blocks; weak scaling.

--impl reference: the reference's CPU implementation of this loop on the host
cores (the reference binary when it is present and runs here, else the oracle's
restatement built with the reference's compiler flags), all host threads, each
step a bounded sample of the same workload.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "samples/s on 1 GB300: mixed-prec batched vs plain FP64 at \u22641e-5 rel err"
UNIT = "samples/s"


def _formula_flops(E, V, K, deformed):
    """Estimated floating-point operations per sample of the reference's algorithm
    (transcendentals once each), for a class the counted table does not hold."""
    n = V - 1
    f = E * (E + 1) + 8 * E + 2 * n ** 3 / 3 + 2 * n ** 3 + V * V + (E + 3) + 2
    if deformed:
        f += 2 * n ** 3 + 4 * n ** 3 + 5 * E * E + 8 * n ** 3 / 3 + 8 * n ** 3 + 8 * E ** 3 / 3 + E + 4
    return f + 4 * K


def _flop_table():
    """profiles/flop_counts.txt: operations per sample counted by running the oracle's
    restatement of the reference's loop with an operation-counting scalar (lines:
    workload E V K deformed add mul div sqrt trans flops cmp samples)."""
    rows = {}
    path = os.path.join(HERE, "profiles", "flop_counts.txt")
    if os.path.exists(path):
        for line in open(path):
            f = line.split()
            if line.startswith("#") or len(f) < 13:
                continue
            rows[(int(f[1]), int(f[2]), bool(int(f[4])))] = (int(f[3]), float(f[10]), f[0])
    return rows


FLOP_TABLE = _flop_table()
_PEAKS = []


def device_peaks(ft):
    """(FP32, FP64) FMA rates of this GPU, probed once per process (outside every timed region)."""
    if not _PEAKS:
        _PEAKS.append(ft.device_peaks())
    return _PEAKS[0]


def algorithmic_flops(E, V, K, deformed):
    """(flops per sample, source): the counted figure of this topology class and regime
    (each further eps order: 8 flops deformed, 2 undeformed), else the estimate."""
    row = FLOP_TABLE.get((E, V, bool(deformed)))
    if row is None:
        return _formula_flops(E, V, K, deformed), "estimate"
    k0, flops, name = row
    return flops + (K - k0) * (8 if deformed else 2), "counted (%s)" % name


def dram_traffic(key):
    """DRAM bytes (read + write) per launch of a kernel from the committed ncu summary
    profiles/dram_traffic.txt (lines: kernel, precision, workload, bytes per launch)."""
    path = os.path.join(HERE, "profiles", "dram_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 4 and not line.startswith("#") and " ".join(parts[:3]) == key:
            return float(parts[3])
    return None


def instructions_per_sample(key):
    """Thread instructions executed per sample by a kernel, from the committed ncu
    summary profiles/instructions.txt (lines: kernel, precision, workload, count)."""
    path = os.path.join(HERE, "profiles", "instructions.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 4 and not line.startswith("#") and " ".join(parts[:3]) == key:
            return float(parts[3])
    return None


def issue_roofline(key, samples_per_s, sm_mhz, sms):
    """Executed thread instructions per second (counted per sample by ncu, times the
    live rate) against the issue capacity: SMs x 4 schedulers x 32 lanes x clock."""
    ips = instructions_per_sample(key)
    if ips is None or not sm_mhz:
        return None
    peak = sms * 4 * 32 * sm_mhz * 1e6 / 1e12
    ach = samples_per_s * ips / 1e12
    return {"achieved": ach, "peak": peak, "unit": "T thread-instructions/s", "frac": ach / peak,
            "instructions_per_sample": ips, "source": "profiles/instructions.txt (ncu, %s)" % key}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"]}
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_rate(inp, seconds, threads, kind_pref=("reference", "port"), n=None):
    """(samples/s, samples, kind) of the reference's CPU loop on this host: the reference
    binary when it is built and runs here, else the restatement built with the
    reference's flags.  n samples, or (n=None) as many as take about `seconds`."""
    ref_bin = os.path.join(HERE, "oracle", "_ref", "feyntrop")
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    if "reference" in kind_pref and os.path.exists(ref_bin):
        try:
            probe = subprocess.run([ref_bin], input=json.dumps(dict(inp, N=20000)), capture_output=True, text=True,
                                   env=env, timeout=120)
            if probe.returncode == 0:
                r0 = 20000 / max(json.loads(probe.stdout)["seconds sampling"], 1e-6)
                if n is None:
                    n = int(max(1e5, min(r0 * seconds, 5e8)))
                out = subprocess.run([ref_bin], input=json.dumps(dict(inp, N=n)), capture_output=True, text=True,
                                     env=env, timeout=600)
                t = json.loads(out.stdout)["seconds sampling"]
                return n / t, n, "reference"
        except (OSError, subprocess.SubprocessError, ValueError, KeyError):
            pass
    sys.path.insert(0, os.path.join(HERE, "tests"))
    import oracle_lib  # the oracle's CPU restatement: the baseline only, never the measured GPU path
    p = oracle_lib.Prepared(inp, fast=True)
    if n is None:
        t0 = time.perf_counter()
        p.integrate(50000, 0, threads)
        r0 = 50000 / (time.perf_counter() - t0)
        n = int(max(1e5, min(r0 * seconds, 5e8)))
    t0 = time.perf_counter()
    p.integrate(n, 0, threads)
    return n / (time.perf_counter() - t0), n, "port"


def batched_section(args, ft, workloads, torch, flush, clocks_sampler, which):
    """The batched form: every integral of a seeded batch in one CUDA graph launch per
    run (ft_batch_*), mixed precision against plain FP64 on the same integrals.

    scan:  4096 box-pentagon kinematic points (masses U[0, 2], invariants U[-10, 10],
           lambda U[0.2, 1], N log-uniform in [1e5, 1e7], Random(3)), about 9e9 samples;
    mixed: 512 triangles, 512 3-loop ladders, 256 4-loop vacuum wheels, 256
           box-pentagons (N log-uniform in [1e5, 1e8], Random(5)), about 2.2e10 samples.
    The FP64 runs use every integral's N times --batch-fp64-scale (the rate does not
    depend on it while the work items outnumber the GPU's block slots).  One warm-up run
    per precision (graph capture), then --batch-steps timed runs with an L2 flush
    between them, timed with CUDA events around the graph launch on its stream."""
    def accept(inp):
        try:
            ft.subgraph_table(inp)
            return True
        except ft.FeyntropError:
            return False

    if which == "scan":
        inputs, redrawn = workloads.box_pentagon_scan(args.batch_count or 4096, seed=3, accept=accept)
        name = ("box-pentagon kinematic scan: 4096 points (7 vertices, 8 edges, D=6, 3 eps orders), masses U[0,2], "
                "invariants U[-10,10], lambda U[0.2,1], N log-uniform [1e5,1e7], Random(3)")
    else:
        inputs, redrawn = workloads.mixed_batch(seed=5, accept=accept)
        if args.batch_count:
            inputs = inputs[:args.batch_count]
        name = ("mixed uneven batch: 512 triangles, 512 3-loop ladders, 256 4-loop vacuum wheels, 256 box-pentagons, "
                "masses U[0,3], N log-uniform [1e5,1e8], Random(5)")
    t0 = time.perf_counter()
    plans = ft.create_plans(inputs)
    t_plans = time.perf_counter() - t0
    Ns = [x["N"] for x in inputs]
    tuned = None
    if not args.no_autotune:
        # one representative per kernel class (topology, eps orders, regime): its mixed
        # launch shape and batch work item, recorded for every batch of the class
        t0 = time.perf_counter()
        tuned = {}
        for p, x in zip(plans, inputs):
            cls = "E%d V%d K%d %s %s" % (p.E, p.V, p.K, "deformed" if p.info["deformed"] else "undeformed",
                                         [e[0] for e in x["graph"]])
            if cls not in tuned:
                r = p.autotune(ft.MIXED)
                tuned[cls] = {k: r[k] for k in ("block", "min_blocks_per_sm", "variant", "batch_chunk",
                                                "samples_per_second", "default_samples_per_second",
                                                "batch_samples_per_second")}
        tuned = {"classes": tuned, "seconds": time.perf_counter() - t0}
    fp32_peak, fp64_peak = device_peaks(ft)
    fl = [algorithmic_flops(p.E, p.V, p.K, bool(p.info["deformed"])) for p in plans]
    flops, flop_src = [f for f, _ in fl], [s_ for _, s_ in fl]
    stream = torch.cuda.Stream()
    out = {"workload": name, "integrals": len(plans), "redrawn": redrawn, "samples_per_run": sum(Ns),
           "seconds_preprocessing_all": t_plans, "autotune": tuned}
    rates = {}
    for prec, scale, tag in ((ft.MIXED, 1.0, "mixed"), (ft.FP64, args.batch_fp64_scale, "plain_fp64")):
        t0 = time.perf_counter()
        b = ft.Batch(plans, prec)
        t_create = time.perf_counter() - t0
        n = [max(1, int(x * scale)) for x in Ns]
        times, res = [], None
        with clocks_sampler() as clk:
            for step in range(1 + args.batch_steps):
                flush.fill_(float(step))
                torch.cuda.synchronize()
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
                res = b.run(n, seeds=step, stream=stream.cuda_stream)
                ev1.record(stream)
                ev1.synchronize()
                if step >= 1:
                    times.append(ev0.elapsed_time(ev1))
        info = b.info()
        ms = sum(times) / len(times)
        rates[tag] = sum(n) / (ms * 1e-3)
        tf = sum(f * k for f, k in zip(flops, n)) / (ms * 1e-3) / 1e12
        peak = fp32_peak if prec == ft.MIXED else fp64_peak
        out[tag] = {"value": rates[tag], "unit": UNIT, "ms_per_run": ms, "runs": len(times),
                    "sample_scale": scale, "samples_per_run": sum(n), "classes": info["num_classes"],
                    "kernel_launches_per_run": info["kernel_launches"], "graph_launches_per_run": 1,
                    "graph_captures": info["graph_captures"], "work_items": info["work_items"],
                    "seconds_batch_create": t_create, "clocks": clk.summary(),
                    "roofline": {"bound": "fp32" if prec == ft.MIXED else "fp64", "achieved": tf, "peak": peak,
                                 "unit": "TFLOP/s", "frac": tf / peak,
                                 "flops_per_sample_mean": sum(f * k for f, k in zip(flops, n)) / sum(n),
                                 "flops_source": sorted(set(flop_src))}}
        if prec == ft.MIXED:
            out[tag]["fp64_fallback_rate"] = sum(r["fp64_fallback"] for r in res) / sum(n)
            out["e2e_mixed"] = {"value": sum(n) / (t_plans + t_create + ms * 1e-3), "unit": UNIT,
                                "includes": "host preprocessing of every integral, batch creation, one run"}
        b.close()
    out["mixed_over_fp64"] = rates["mixed"] / rates["plain_fp64"]
    out["mixed_over_fp64_samples_per_run"] = {"mixed": out["mixed"]["samples_per_run"],
                                              "plain_fp64": out["plain_fp64"]["samples_per_run"],
                                              "note": "the FP64 arm runs every integral's N x %g (the rate does not "
                                                      "depend on N while work items outnumber the GPU's block slots)"
                                                      % args.batch_fp64_scale}
    # the CPU path on a bounded, evenly spaced subset of the same integrals
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        pick = list(range(0, len(inputs), max(1, len(inputs) // 8)))[:8]
        tot_n = tot_t = 0.0
        kind = None
        for i in pick:
            v, n, kind = cpu_rate(inputs[i], args.cpu_seconds / len(pick), threads)
            tot_n += n
            tot_t += n / v
        out["cpu_baseline"] = {"value": tot_n / tot_t, "unit": UNIT, "cores": threads, "kind": kind,
                               "sample": "integrals %s of the batch, %d samples in total, all host threads"
                                         % (pick, int(tot_n))}
        out["mixed_over_cpu"] = rates["mixed"] / out["cpu_baseline"]["value"]
    # per-sample error of the mixed form against the FP64 form, per kernel class: its
    # first four integrals in the batch's order, 32768 samples each
    by_class = {}
    for p, x in zip(plans, inputs):
        cls = "E%d V%d K%d %s" % (p.E, p.V, p.K, "deformed" if p.info["deformed"] else "undeformed")
        if len(by_class.setdefault(cls, [])) < 4:
            by_class[cls].append(p)
    out["per_sample_error"] = {cls: sample_error(ft, ps, len(ps) << 15) for cls, ps in sorted(by_class.items())}
    worst = max(by_class, key=lambda c: out["per_sample_error"][c]["max"])
    out["per_sample_error_max"] = {"class": worst, "max": out["per_sample_error"][worst]["max"],
                                   "frac_above_1e-5": max(v["frac_above_1e-5"]
                                                          for v in out["per_sample_error"].values())}
    for p in plans:
        p.close()
    return out


def sample_error(ft, plans, samples):
    """Per-sample relative error of the mixed form against the plain-FP64 GPU form on the
    same samples (seed 0; `samples` split over the plans): max over eps orders and Re/Im,
    relative to the sample's largest component; samples the FP64 form drops are left out."""
    import numpy as np
    errs = []
    for p in plans:
        n = max(1, samples // len(plans))
        rm = p.records(n, seed=0, precision=ft.MIXED)
        r6 = p.records(n, seed=0, precision=ft.FP64)
        ok = (r6["flags"] & 1) == 0
        scale = np.abs(r6["R"][ok]).max(axis=1)
        errs.append(np.abs(rm["R"][ok] - r6["R"][ok]).max(axis=1) / np.where(scale > 0, scale, 1.0))
    e = np.concatenate(errs)
    return {"samples": int(e.size), "max": float(e.max()), "mean": float(e.mean()),
            "p99.9": float(np.quantile(e, 0.999)), "frac_above_1e-5": float((e > 1e-5).mean()),
            "against": "the plain-FP64 GPU form (itself checked against the CPU oracle in tests), seed 0, "
                       "%d integral(s)" % len(plans)}


def configs_section(args, ft, workloads, torch, flush):
    """The other single-integral configurations, each timed like the headline step
    (one warm-up, two timed integrations with CUDA events on the integration stream,
    L2 flushed between them), mixed and plain FP64:
      K4:   complete graph K4, Euclidean, masses 0..5, 3 eps orders, N = 1e7;
      cube: 5-loop 2-point cube graph (8 vertices, 12 edges), Euclidean, 4 eps orders,
            N = 1e9 in both forms."""
    stream = torch.cuda.Stream()
    fp32_peak, fp64_peak = device_peaks(ft)
    out = {}
    for name, inp, n_mixed, n_fp64 in (("K4", workloads.k4_euclidean(), 10 ** 7, 10 ** 7),
                                      ("cube", workloads.cube_propagator(), 10 ** 9, 10 ** 9)):
        plan = ft.Plan(inp)
        entry = {"workload": name, "samples_mixed": n_mixed, "samples_fp64": n_fp64}
        for prec, n, tag in ((ft.MIXED, n_mixed, "mixed"), (ft.FP64, n_fp64, "plain_fp64")):
            times, res = [], None
            with torch.cuda.stream(stream):
                for step in range(3):
                    flush.fill_(float(step))
                    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    ev0.record(stream)
                    res = plan.integrate(n, seed=step, precision=prec, stream=stream.cuda_stream)
                    ev1.record(stream)
                    ev1.synchronize()
                    if step >= 1:
                        times.append(ev0.elapsed_time(ev1))
            ms = sum(times) / len(times)
            flops, src = algorithmic_flops(plan.E, plan.V, plan.K, bool(plan.info["deformed"]))
            tf = flops * n / (ms * 1e-3) / 1e12
            peak = fp32_peak if prec == ft.MIXED else fp64_peak
            entry[tag] = {"value": n / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
                          "fp64_fallback_rate": res["fp64_fallback"] / n, "integral": res["integral"],
                          "roofline": {"bound": "fp32" if prec == ft.MIXED else "fp64", "achieved": tf, "peak": peak,
                                       "unit": "TFLOP/s", "frac": tf / peak, "flops_per_sample": flops,
                                       "flops_source": src}}
        entry["mixed_over_fp64"] = entry["mixed"]["value"] / entry["plain_fp64"]["value"]
        entry["per_sample_error"] = sample_error(ft, [plan], 1 << 19)
        out[name] = entry
        plan.close()
    return out


def lambda_section(ft, workloads, N):
    """The deformation parameter of the double box chosen by pilot runs
    (ft.choose_lambda), and the time to a 1e-4 relative error of Re I0 at the chosen
    lambda against the benchmark's lambda = 0.5 (same rate measurement: one timed
    mixed integration of N samples at each)."""
    inp = workloads.double_box(N=1000)
    (lam, rel, table), = ft.choose_lambda([inp], candidates=(0.05, 0.1, 0.2, 0.3, 0.5, 0.8), pilot=10 ** 6)
    out = {"candidates_relative_error": {str(k): v for k, v in table.items()}, "chosen": lam}
    for tag, l in (("chosen", lam), ("benchmark", 0.5)):
        p = ft.Plan(dict(inp, **{"lambda": l}))
        p.integrate(N // 10, seed=0, precision=ft.MIXED)
        r = p.integrate(N, seed=1, precision=ft.MIXED)
        rate = N / (r["kernel_ms"] * 1e-3)
        (re, dre), (im, dim) = r["integral"][0]
        spread = dre * math.sqrt(N)
        target = 1e-4 * abs(re)
        out[tag] = {"lambda": l, "integral_eps0": [[re, dre], [im, dim]], "samples_per_second": rate,
                    "time_to_1e-4_relative_s": (spread / target) ** 2 / rate if target > 0 else None}
        p.close()
    c, b_ = out["chosen"]["time_to_1e-4_relative_s"], out["benchmark"]["time_to_1e-4_relative_s"]
    out["speedup_time_to_target"] = b_ / c if (b_ and c) else None
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from feyntrop_gb300 import workloads
    inp = workloads.double_box(N=args.samples)
    threads = os.cpu_count() or 1
    # the first warm-up step sizes the per-step sample (about --ref-seconds of CPU work);
    # every later step runs exactly that many samples, and a step's time is theirs
    _, nsample, kind = cpu_rate(inp, args.ref_seconds, threads)
    secs = []
    for step in range(max(0, args.warmup - 1) + args.steps):
        v, _, kind = cpu_rate(inp, args.ref_seconds, threads, n=nsample)
        if step >= max(0, args.warmup - 1):
            secs.append(nsample / v)
    value = nsample * len(secs) / sum(secs)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum(secs) / len(secs) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded double-box kinematics)",
        "config": {"workload": "double box, Minkowski, lambda=0.5, 2 eps orders, N=%d per step: a bounded sample "
                               "(about %.0f s of all host cores) of the N=%d workload, the same stream"
                               % (nsample, args.ref_seconds, args.samples),
                   "host_threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": "%d samples of the double-box stream per step (seed 0, samples [0, N))"
                                   % nsample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--samples", type=int, default=10 ** 8)
    ap.add_argument("--ref-seconds", type=float, default=4.0)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kernel-only", action="store_true",
                    help="only the timed sampling steps (for profiler captures); prints a reduced line")
    ap.add_argument("--workload", default="double_box", choices=["double_box", "cube", "ladder_mink", "box_pentagon"],
                    help="with --kernel-only: the integral of the timed steps (profiler captures of other classes)")
    ap.add_argument("--batched", default="both", choices=["both", "scan", "mixed", "none"],
                    help="the batched form's workloads (one GPU runs them, rank 0 reports them)")
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--no-configs", action="store_true", help="skip the K4 and cube configurations")
    ap.add_argument("--batch-count", type=int, default=0,
                    help="only the first n integrals of the batch (profiler captures); 0: all")
    ap.add_argument("--batch-only", action="store_true",
                    help="only the batched form (profiler captures); prints its object alone")
    ap.add_argument("--batch-fp64-scale", type=float, default=1 / 16)
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched section: keep the default launch shapes instead of autotuning each kernel class")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import feyntrop_gb300 as ft
    from feyntrop_gb300 import workloads

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        dist = None

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    if args.batch_only:
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        which = ["scan", "mixed"] if args.batched == "both" else [args.batched]
        print(json.dumps({w: batched_section(args, ft, workloads, torch, flush, lambda: ClockSampler(local), w)
                          for w in which}), flush=True)
        return
    N = args.samples
    if args.workload != "double_box" and not args.kernel_only:
        raise SystemExit("--workload other than double_box needs --kernel-only (the headline is the double box)")
    def accept(x):
        try:
            ft.subgraph_table(x)
            return True
        except ft.FeyntropError:
            return False

    if args.workload == "cube":
        inp = workloads.cube_propagator(N=N)
    elif args.workload == "ladder_mink":
        # a Minkowski 3-loop ladder drawn as in the mixed batch (Random(5): masses U[0, 3],
        # s U[8, 20], t U[-6, -1], lambda 0.5; the second ladder drawn, the first Minkowski one)
        inp = [x for x in workloads.mixed_batch(seed=5, counts=(0, 2, 0, 0), accept=accept)[0] if x["lambda"] != 0][0]
    elif args.workload == "box_pentagon":
        inp = workloads.box_pentagon_scan(1, seed=3, accept=accept)[0][0]
    else:
        inp = workloads.double_box(N=N)
    plan = ft.Plan(inp)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed_steps(precision, K, W, tag):
        res = []
        times = []
        with torch.cuda.stream(stream):
            for s in range(W + K):
                flush.fill_(float(s))
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
                r = plan.integrate(N, seed=s, precision=precision, first_sample=rank * N,
                                   stream=stream.cuda_stream)
                ev1.record(stream)
                ev1.synchronize()
                if s >= W:
                    times.append(ev0.elapsed_time(ev1))
                    res.append(r)
        return times, res

    # warm-up (kernel compilation, skip matrices) outside any timing
    timed_steps(ft.MIXED, 0, args.warmup, "warm")
    timed_steps(ft.FP64, 0, 1, "warm")
    barrier()
    with ClockSampler(local) as clk:
        barrier()
        t_mixed, r_mixed = timed_steps(ft.MIXED, args.steps, 0, "mixed")
        barrier()
    clocks = clk.summary()
    barrier()
    fp64_steps = max(2, min(args.steps, 3))
    t_fp64, r_fp64 = timed_steps(ft.FP64, fp64_steps, 0, "fp64")
    barrier()

    ms_mixed = sum(t_mixed) / len(t_mixed)
    ms_fp64 = sum(t_fp64) / len(t_fp64)
    if args.kernel_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": N * world / (ms_mixed * 1e-3), "unit": UNIT,
                              "ms_per_step": ms_mixed, "fp64_ms_per_step": ms_fp64, "kernel_only": True}))
        return
    if dist:
        t = torch.tensor([ms_mixed, ms_fp64], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_mixed, ms_fp64 = t.tolist()
    value = N * world / (ms_mixed * 1e-3)
    value64 = N * world / (ms_fp64 * 1e-3)

    # per-sample error of the mixed form against the FP64 form on the same samples
    # (2^20 of them: the tail above 1e-5 is a few per million)
    err_stats = sample_error(ft, [plan], 1 << 20)

    # end to end through the public API: plan (host preprocessing + upload), integrate, read back
    barrier()
    e2e_times = []
    h2d = d2h = 0
    for s in range(args.steps):
        t0 = time.perf_counter()
        p2 = ft.Plan(inp)
        r = p2.integrate(N, seed=100 + s, precision=ft.MIXED, first_sample=rank * N)
        e2e_times.append(time.perf_counter() - t0)
        h2d = p2.info["table_bytes"] + 8 * (8 + 2 * p2.E + 64)
        d2h = 8 * (8 * p2.K + 8) + 4
        p2.close()
    e2e_s = sum(e2e_times) / len(e2e_times)
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = t.item()

    # merged result over ranks (moments are additive)
    from feyntrop_gb300 import shard
    moments = r_mixed[-1]["moments"]
    if dist:
        allm = [None] * world
        dist.all_gather_object(allm, moments)
        moments = shard.merge_moments(allm)
    integral = ft.finalize_moments(moments, plan.K, real_only=not plan.info["deformed"])

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    fp32_peak, fp64_peak = device_peaks(ft)
    flops, flops_src = algorithmic_flops(plan.E, plan.V, plan.K, bool(plan.info["deformed"]))
    launches = sum(r["kernel_launches"] for r in r_mixed)
    fallback = sum(r["fp64_fallback"] for r in r_mixed) / (N * len(r_mixed))
    acc0 = integral[0][0][1]
    sigma1 = acc0 * math.sqrt(N * world)
    target = 1e-4 * abs(integral[0][0][0])
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        threads = os.cpu_count() or 1
        v, nsample, kind = cpu_rate(inp, args.cpu_seconds, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": "%d samples of the double-box workload (same stream), all host threads" % nsample}
    traffic = dram_traffic("ft_sample mixed double_box")
    # per-launch duration of the sampling kernels (events inside ft_integrate around
    # ft_sample and its FP64 pass, on the integration stream)
    kms = sum(r["kernel_ms"] for r in r_mixed) / len(r_mixed)
    achieved = flops * N / (kms * 1e-3) / 1e12
    hbm = None
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
        if traffic:
            gbs = traffic / (kms * 1e-3) / 1e9
            hbm = {"achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": gbs / peaks["hbm_gbs"],
                   "peak_source": "measured (MEASURED_PEAKS.json)"}
    except (OSError, ValueError, KeyError):
        pass
    batched = None
    if args.batched != "none" and rank == 0:
        which = ["scan", "mixed"] if args.batched == "both" else [args.batched]
        batched = {w: batched_section(args, ft, workloads, torch, flush, lambda: ClockSampler(local), w)
                   for w in which}
    other = configs_section(args, ft, workloads, torch, flush) if (rank == 0 and not args.no_configs) else None
    lam = lambda_section(ft, workloads, 10 ** 8) if (rank == 0 and not args.no_configs) else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 integrand, f64 sector decisions and fallback",
        "data": "synthetic (seeded double-box kinematics, Random(1))",
        "config": {"workload": "double box (6 vertices, 7 edges), Minkowski, lambda=0.5, D=4, 2 eps orders, "
                               "N=%d samples per step per GPU" % N,
                   "precision": "mixed", "parallelism": "sample blocks of one stream per GPU",
                   "l2": "flushed between steps (256 MiB write), per-step CUDA events on the kernels' stream"},
        "plain_fp64": {"value": value64, "ms_per_step": ms_fp64, "steps": len(t_fp64),
                       "roofline": {"bound": "fp64", "achieved": flops * value64 / world / 1e12,
                                    "peak": fp64_peak, "unit": "TFLOP/s",
                                    "frac": flops * value64 / world / 1e12 / fp64_peak}},
        "mixed_over_fp64": value / value64,
        "per_sample_error": err_stats,
        "fp64_fallback_rate": fallback,
        "integral": integral,
        "time_to_target_sigma_s": {"target": "1e-4 * |Re I0|", "mixed": (sigma1 / target) ** 2 / value,
                                   "fp64": (sigma1 / target) ** 2 / value64},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": traffic,
                     "hbm": hbm,
                     "issue": issue_roofline("ft_sample mixed double_box", N / (kms * 1e-3),
                                             clocks.get("sm_mhz"),
                                             torch.cuda.get_device_properties(local).multi_processor_count),
                     "flops_per_sample": flops,
                     "note": "algorithmic flops per sample %.0f of the reference's loop, %s: the oracle's "
                             "restatement run with an operation-counting scalar (profiles/flop_counts.txt) x samples "
                             "per launch / the sampling kernels' CUDA-event time (ft_sample + its FP64 pass, %.2f ms); "
                             "peak = FP32 FMA issue rate measured live by an FMA-chain probe (FP64: %.2f TFLOP/s). "
                             "Neither HBM nor tensor cores bound this path: see hbm" % (flops, flops_src, kms,
                                                                                         fp64_peak)},
        "e2e": {"value": N * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks,
        "cpu_baseline": cpu,
        "batched": batched,
        "other_configs": other,
        "lambda_choice": lam,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
