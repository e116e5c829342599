#!/usr/bin/env python
"""Benchmark of the likelihood + branch-length-gradient path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload batched-hky-g4|gtr-g4|restriction|restriction-g4-bd|protein-g4]

One step = one logL + gradient evaluation of the whole workload (every instance,
every site, every rate category) after a new set of branch lengths, i.e. one
leapfrog step of a sampler.  Metric: site-node updates/s, units = sum over
instances of (N_i - 1) * S_i * C.

Default workload: 256 independent HKY+G4 instances of uneven size in one launch
(T ~ logU[16, 1024] taxa, S ~ logU[500, 50000] sites, kappa ~ LogNormal(1, 0.5)),
FP32-scaled path, compared with the plain FP64 GPU path on the same inputs.

value: device-resident inputs (branch lengths already in HBM), each evaluation
replayed as one captured CUDA graph, CUDA events on the engine's stream around
each step, L2 flushed (512 MB write) between steps outside the events; per-kernel
times come from a separate pass with the engine's own events.  e2e: the same step through the C ABI with host buffers (branch
lengths in, ll and gradient out, copies inside the timed region).
--impl reference: the CPU restatement of the reference's loops (FP64, OpenMP, all
host cores) on a bounded sample of the same workload each step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "mcphylo.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "logL+grad site-node updates/s, FP32-scaled vs plain FP64 GPU at ≤1e-6 rel err"
UNIT = "site-node updates/s"


# ----------------------------------------------------------------------------- workloads
def make_workload(name, workers, site_scale=1.0):
    from mcphylo_gb300 import simulate
    if name == "batched-hky-g4":
        insts = simulate.hky_batch(seed=4, n=256, workers=workers, scale=site_scale)
        cfg = {"workload": "batched-hky-g4", "instances": 256, "taxa": "logU[16,1024]",
               "sites": "logU[500,50000]", "model": "HKY+G4 (shape 0.5), kappa~LogNormal(1,0.5)",
               "states": 4, "rates": 4}
    elif name == "gtr-g4":
        insts = [simulate.gtr_gamma(S=max(1, int(100_000 * site_scale)), with_weights=True)]
        cfg = {"workload": "gtr-g4", "taxa": 128, "sites": "100,000 patterns",
               "pattern_weights": "Poisson(1)+1", "model": "GTR+G4 (shape 0.5)",
               "states": 4, "rates": 4}
    elif name == "restriction":
        insts = [simulate.restriction_small(S=max(1, int(1000 * site_scale)))]
        cfg = {"workload": "restriction", "taxa": 32, "sites": 1000, "model": "Restriction",
               "states": 2, "rates": 1}
    elif name == "restriction-g4-bd":
        insts = [simulate.restriction_gamma_bd(S=max(1, int(20_000 * site_scale)))]
        cfg = {"workload": "restriction-g4-bd", "taxa": 512, "sites": 20_000,
               "model": "Restriction+G4 (shape 1)", "states": 2, "rates": 4}
    elif name == "protein-g4":
        insts = [simulate.protein_gamma(S=max(1, int(50_000 * site_scale)))]
        cfg = {"workload": "protein-g4", "taxa": 256, "sites": 50_000,
               "model": "GTR20+G4 (shape 0.5)", "states": 20, "rates": 4}
    else:
        raise SystemExit(f"unknown workload {name}")
    if site_scale != 1.0:
        cfg["site_scale"] = site_scale   # a profiling case, not the benchmark
    cfg["units_per_step"] = int(sum(i.units() for i in insts))
    return insts, cfg


def make_engine(insts, precision, tiles=None, sweep="auto"):
    import mcphylo_gb300 as mp
    e = mp.Engine(insts[0].K, len(insts[0].rates), precision, n_instances=len(insts))
    if tiles:
        e.set_tiles(*tiles)
    if precision in ("f32", "f64"):
        e.set_sweep(sweep)
    for i, b in enumerate(insts):
        e.set_tree(b.parent, b.blen, i)
        e.set_codes(b.codes, b.leaf_nums, i)
        if b.weights is not None:
            e.set_weights(b.weights, i)
        e.set_model(b.U, b.D, b.Uinv, b.mu, b.pi, b.rates, i)
    return e


def tc_algorithmic_bytes(insts, grad=True, prec="tf32"):
    """Bytes the tensor-core kernel must move per evaluation: every post-order partial
    of an internal non-root step written once (as an operand tile, KD entries per
    site, 4 bytes in TF32, 2 in BF16, 8 in split TF32: value and residual) and read
    once by the gradient sweep, the leaf state codes read once (4 bytes), the per-item
    gradient partials written once."""
    import mcphylo_gb300 as mp
    total = 0
    step = 16 if prec == "bf16" else 8
    esz = {"bf16": 2, "tf32": 4, "tf32x3": 8}[prec]
    for b in insts:
        KD = (b.K + step - 1) // step * step
        info = mp.schedule_info(b.parent)
        C = len(b.rates)
        blocks = -(-b.S // 128)
        lanes = blocks * 128 * C
        total += len(b.leaf_nums) * b.S * 4
        if grad:
            total += 2 * lanes * (info["internal"] - 1) * KD * esz
            total += C * blocks * (b.N - 1) * 4
        else:
            total += lanes * (info["internal"] - 1) * KD * esz
    return total


def algorithmic_bytes(insts, spt, real_bytes, grad=True):
    """Bytes the fused kernel must move per evaluation: every post-order partial of
    an internal non-root step written once and read once (gradient mode only), the
    leaf state codes read once, the per-item gradient partials written once."""
    import mcphylo_gb300 as mp
    total = 0
    K = insts[0].K
    Kp = 2 if K <= 2 else 4 if K <= 4 else 8 if K <= 8 else 20 if K <= 20 else 32
    code_b = 1 if Kp <= 8 else 4
    for b in insts:
        info = mp.schedule_info(b.parent)
        C = len(b.rates)
        lanes = b.S * C
        blocks = -(-b.S // (32 * spt))
        total += len(b.leaf_nums) * b.S * code_b
        if grad:
            total += 2 * lanes * (info["internal"] - 1) * Kp * real_bytes
            total += C * blocks * (b.N - 1) * real_bytes
    return total


def level_algorithmic_bytes(insts, real_bytes, grad=True):
    """Bytes the level-synchronous sweep must move per evaluation: its partials stay
    in shared memory, so the leaf state codes read once, the step records read once
    per (instance, rate) and the per-item gradient partials written once."""
    K = insts[0].K
    Kp = 2 if K <= 2 else 4 if K <= 4 else 8
    rec = 48 + 4 * (Kp + 1) * Kp * real_bytes
    total = 0
    for b in insts:
        C = len(b.rates)
        J = len(b.leaf_nums) - 1
        total += len(b.leaf_nums) * b.S * 1 + C * J * rec
        if grad:
            total += C * (-(-b.S // 32)) * (b.N - 1) * real_bytes
    return total


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, index=0):
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
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for ln in open(self.path):
                f = [x.strip() for x in ln.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------------------- CPU sample
def oracle_windows(insts, units_budget, window=2000):
    """The bounded CPU sample of a workload, the same for the reference arm and the
    cpu_baseline leg: windows of at most ``window`` sites, one per instance, the
    instances taken at a fixed stride through the workload (so a batched workload's
    sample spans its range of tree and alignment sizes), until ``units_budget``
    units; a single-instance workload gives consecutive windows of its sites.
    Returns [(oracle tree, site tensor, instance window)]."""
    from oracle import pyoracle as O
    from mcphylo_gb300 import simulate
    n = len(insts)
    stride = 97 if n > 97 and n % 97 else 1
    order = [(i * stride) % n for i in range(n)]
    out, units = [], 0
    rounds = 1 if n > 1 else max(1, -(-insts[0].S // window))
    for r in range(rounds):
        for ii in order:
            b = insts[ii]
            s0 = r * window
            sub = simulate.Instance(b.tree, b.parent, b.blen, b.leaf_nums,
                                    b.codes[:, s0:s0 + window], b.U, b.D, b.Uinv, b.mu,
                                    b.pi, b.rates)
            out.append((O.tree_from_parent(sub.parent, sub.blen), sub.tensor(), sub))
            units += sub.units()
            if units >= units_budget:
                return out
    return out


def cpu_leg(args):
    """The cpu_baseline leg of the GPU arm: the reference arm (the oracle on its
    bounded sample, oracle_windows) run as a child process, so that it times the same
    code on the same windows in a process whose cores no GPU-side runtime (torch's
    thread pool, the clock sampler) shares.  Returns the reference arm's JSON line."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--workload",
           args.workload, "--steps", str(args.cpu_steps), "--warmup", "3", "--ref-units",
           str(args.ref_units)]
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    p = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=1800,
                       cwd=os.path.dirname(os.path.abspath(__file__)))
    if p.returncode != 0:
        raise RuntimeError("cpu_baseline leg failed: " + p.stderr[-2000:])
    return json.loads(p.stdout.strip().splitlines()[-1])


# ----------------------------------------------------------------------------- reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return 0
    insts, cfg = make_workload(args.workload, workers=min(16, os.cpu_count() or 1))
    from oracle import pyoracle as O
    O.lib()
    # one step = the oracle's logL + gradient on a fixed bounded sample (the same
    # windows as the cpu_baseline leg of the GPU arm)
    sample = oracle_windows(insts, args.ref_units)
    units = sum(s[2].units() for s in sample)

    def step():
        for t, x, s in sample:
            O.gradlogpdf(t, x, s.pi, (s.U, s.D, s.Uinv, s.mu), s.rates)

    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    ms = 1e3 * statistics.mean(times)
    v = units / (ms / 1e3)
    desc = (f"{len(sample)} windows of <=2000 sites (one per instance, instances at a fixed "
            f"stride through the workload), {units} units per step")
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded simulation)", "config": cfg,
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
                            "sample": desc},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "the reference is Julia and cannot run here; this is the C/OpenMP FP64 "
                   "restatement of its loops (oracle/oracle.c)"}
    print(json.dumps(out), flush=True)
    return 0


# ----------------------------------------------------------------------------- NUTS ESS/s
NUTS_PRIOR = (1.0, 1.0, 0.1, 1.0)     # CompoundDirichlet(alpha, a, beta, c)


def _oracle_posterior(inst, prior):
    from oracle import pyoracle as O
    x = np.asfortranarray(inst.tensor())
    model = (inst.U, inst.D, inst.Uinv, inst.mu)
    timer = {"grad_s": 0.0, "grad_n": 0, "logf_s": 0.0, "logf_n": 0}

    def lfg(p, b):
        t0 = time.perf_counter()
        ll, g = O.gradlogpdf(O.tree_from_parent(p, b), x, inst.pi, model, inst.rates)
        timer["grad_s"] += time.perf_counter() - t0
        timer["grad_n"] += 1
        lp, gp = prior.logpdf_grad(p, b)
        return ll + lp, g + gp

    def lf(p, b):
        t0 = time.perf_counter()
        ll = O.logpdf(O.tree_from_parent(p, b), x, inst.pi, model, inst.rates)
        timer["logf_s"] += time.perf_counter() - t0
        timer["logf_n"] += 1
        return ll + prior.logpdf_grad(p, b)[0]

    return lfg, lf, timer


def _chain_summary(ch):
    e = ch.ess()
    ess_min = min(e["logf"], e["tree_length"])
    return {"ess_per_s": ess_min / ch.seconds, "ess": e, "seconds": round(ch.seconds, 3),
            "iterations": len(ch.logf), "grad_evals": ch.grad_evals,
            "logf_evals": ch.logf_evals, "mean_depth": float(np.mean(ch.depth)),
            "epsilon": ch.epsilon, "nni_moves": int(np.sum(ch.nni_moves)),
            "ms_per_grad_eval": 1e3 * ch.seconds / max(ch.grad_evals, 1),
            "adapt_seconds": round(ch.adapt_seconds, 3)}


def run_nuts(args):
    """NUTS ESS/s: one PNUTS chain over the branch lengths of one workload (the
    likelihood times a CompoundDirichlet(1, 1, 0.1, 1) tree prior), driven by the
    FP32 engine, by the FP64 engine and by the CPU oracle with the same seed.
    ESS = min over (log posterior, tree length) of min((SD / MCSE_bm)^2, n),
    batch size 100, over the post-adaptation draws; time = wall clock of those
    iterations (host sampler + evaluations)."""
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from mcphylo_gb300 import pnuts as P
    insts, cfg = make_workload(args.workload, workers=min(16, os.cpu_count() or 1))
    if len(insts) != 1:
        raise SystemExit("--mode nuts runs on a single-tree workload")
    inst = insts[0]
    prior = P.CompoundDirichlet(*NUTS_PRIOR)
    # the benchmark's chain lengths: 1000 iterations on the 32-taxon restriction
    # workload, 2000 on the 512-taxon birth-death one
    n_iter = args.nuts_iter or (2000 if args.workload == "restriction-g4-bd" else 1000)
    n_adapt = args.nuts_adapt
    # --nuts-plus-forward: the variant whose plus end starts with direction +1 (not the
    # reference's sampler), FP32 engine only, to measure what the quirk costs
    variant = bool(args.nuts_plus_forward)
    res = {}
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for prec in (("f32",) if variant else ("f32", "f64")):
            post = P.engine_posterior(inst.parent, inst.blen, inst.codes, inst.leaf_nums,
                                      (inst.U, inst.D, inst.Uinv, inst.mu), inst.pi, inst.rates,
                                      prior, precision=prec)
            spent = {"s": 0.0, "n": 0}

            def timed(fn):
                def call(p, b):
                    t0 = time.perf_counter()
                    try:
                        return fn(p, b)
                    finally:
                        spent["s"] += time.perf_counter() - t0
                        spent["n"] += 1
                return call

            ch = P.run_chain(inst.parent, inst.blen, timed(post.logfgrad), timed(post.logf),
                             n_iter=n_iter, n_adapt=n_adapt, seed=args.nuts_seed,
                             target=args.nuts_target, plus_end_forward=variant)
            res[prec] = _chain_summary(ch)
            res[prec]["set_tree_calls"] = post.n_set_tree
            # host time of the sampling iterations: wall time minus the evaluations
            per_eval = spent["s"] / max(spent["n"], 1)
            res[prec]["host_seconds"] = max(
                ch.seconds - per_eval * (ch.grad_evals + ch.logf_evals), 0.0)
            # one posterior evaluation as the sampler calls it (wall, host API with the
            # prior) against the device time of the engine's evaluation (CUDA events)
            res[prec]["ms_per_eval_call"] = 1e3 * per_eval
            e = post.eng
            e.enable_timing(True)
            dev = []
            for _ in range(30):
                e.logpdf_grad()
                t3 = e.timing()
                dev.append(t3["build_p_ms"] + t3["prune_ms"] + t3["reduce_ms"])
            e.enable_timing(False)
            res[prec]["device_ms_per_grad_eval"] = statistics.median(dev[5:])
            res[prec]["launches_per_eval"] = e.counts()["launches"]
    clocks = clk.summary()
    if variant:
        out = {"metric": "NUTS ESS/s (PNUTS over branch lengths)", "value": res["f32"]["ess_per_s"],
               "unit": "effective samples/s", "n_gpus": 1, "higher_is_better": True,
               "dtype": "f32", "data": "synthetic (seeded simulation)",
               "variant": "plus end starts with direction +1 (not the reference's sampler)",
               "config": dict(cfg, iterations=n_iter, adaptation=n_adapt,
                              prior="CompoundDirichlet(1,1,0.1,1)", target=args.nuts_target,
                              tree_depth=10, seed=args.nuts_seed),
               "nuts": {"f32": res["f32"]}, "clocks": clocks}
        print(json.dumps(out), flush=True)
        return 0
    # CPU: the oracle drives the same sampler.  With the same seed its chain retraces
    # the FP64 engine's (the decisions agree), so where a full run does not fit the
    # time budget, its time is the FP64 chain's evaluation counts at the oracle's
    # measured cost per evaluation plus the FP64 chain's host time.
    from oracle import pyoracle as O
    O.lib()
    lfg, lf, timer = _oracle_posterior(inst, prior)
    lfg(inst.parent, inst.blen)
    per_grad = timer["grad_s"]
    f64 = res["f64"]
    evals_per_iter = (f64["grad_evals"] + f64["logf_evals"]) / max(n_iter, 1)
    est_total = (n_iter + n_adapt) * evals_per_iter * per_grad
    if est_total <= args.cpu_seconds * 4:
        ch = P.run_chain(inst.parent, inst.blen, lfg, lf, n_iter=n_iter, n_adapt=n_adapt,
                         seed=args.nuts_seed, target=args.nuts_target)
        cpu = _chain_summary(ch)
        cpu["kind"] = "port, full chain"
    else:
        timer.update(grad_s=0.0, grad_n=0, logf_s=0.0, logf_n=0)
        while timer["grad_s"] + timer["logf_s"] < args.cpu_seconds:
            lfg(inst.parent, inst.blen)
            lf(inst.parent, inst.blen)
        g_s = timer["grad_s"] / timer["grad_n"]
        f_s = timer["logf_s"] / timer["logf_n"]
        secs = f64["grad_evals"] * g_s + f64["logf_evals"] * f_s + f64["host_seconds"]
        ess_min = min(f64["ess"]["logf"], f64["ess"]["tree_length"])
        cpu = {"ess_per_s": ess_min / secs, "seconds": round(secs, 3),
               "oracle_grad_s": g_s, "oracle_logf_s": f_s,
               "kind": "port, estimated: the FP64 chain's evaluation counts x the oracle's "
                       "time per evaluation (%d grad, %d logf evaluations timed) + the FP64 "
                       "chain's wall time" % (timer["grad_n"], timer["logf_n"])}
    cpu["cores"] = O.num_threads()
    out = {"metric": "NUTS ESS/s (PNUTS over branch lengths)", "value": res["f32"]["ess_per_s"],
           "unit": "effective samples/s", "n_gpus": 1, "higher_is_better": True,
           "dtype": "f32", "data": "synthetic (seeded simulation)",
           "config": dict(cfg, iterations=n_iter, adaptation=n_adapt,
                          prior="CompoundDirichlet(1,1,0.1,1)", target=args.nuts_target,
                          tree_depth=10, seed=args.nuts_seed),
           "nuts": {"f32": res["f32"], "f64": res["f64"], "cpu_oracle": cpu},
           "clocks": clocks}
    print(json.dumps(out), flush=True)
    return 0


# ----------------------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world):
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", rank=rank, world_size=world)
    insts, cfg = make_workload(args.workload, workers=min(16, os.cpu_count() or 1),
                               site_scale=args.site_scale)
    units = cfg["units_per_step"]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_kind = "measured" if "hbm_gbs" in peaks else "fallback"

    prec = args.precision
    tc_path = prec in ("tf32", "bf16", "tf32x3")
    if tc_path and insts[0].K < 9:
        raise SystemExit("--precision tf32/bf16/tf32x3 is the dense-state path (K >= 9)")
    if args.tiles == "auto" and args.sweep == "auto" and args.walk == "auto" and not args.rates_per_warp:
        # the library's autotuner: times each sweep and launch shape on this problem
        e = make_engine(insts, prec)
        tiles = e.autotune()
        tune = {"chosen_by": "mcphy_autotune"}
    else:
        tiles = None if args.tiles == "auto" else tuple(int(x) for x in args.tiles.split("x"))
        tune = {"chosen_by": "command line"}
        e = make_engine(insts, prec, tiles, args.sweep)
        if args.rates_per_warp:
            e.set_rates_per_warp(args.rates_per_warp)
        if args.walk == "general":
            e.debug_inject(3)   # the general tree walk (dense / ambiguous leaves) on every instance
        tiles = tiles or (1, 128)
    sweep = e.sweep() if not tc_path else "tensor-core"
    rpw = e.tiles()[2] if not tc_path else 1
    M = len(insts)
    off = e.grad_offsets()
    G = int(off[-1])
    # a dedicated (non-default) stream shared by the engine, the L2 flush and the events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    e.set_stream(stream.cuda_stream)
    e.enable_timing(True)

    # branch-length sets for every step (leapfrog-like multiplicative moves)
    rng = np.random.default_rng(123 + rank)
    base = np.concatenate([b.blen for b in insts])
    nsets = args.warmup + args.steps
    host_sets = [base * np.exp(0.05 * rng.standard_normal(base.shape)) for _ in range(nsets)]
    dev_sets = torch.tensor(np.stack(host_sets), dtype=torch.float64, device="cuda")
    d_ll = torch.zeros(M, dtype=torch.float64, device="cuda")
    d_grad = torch.zeros(G, dtype=torch.float64, device="cuda")
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 512 MB > L2

    def dev_step(eng, k):
        eng.set_all_branch_lengths_device(dev_sets[k % nsets].data_ptr())
        if args.mode == "grad":
            eng.logpdf_grad_device(d_ll.data_ptr(), d_grad.data_ptr())
        else:
            eng.logpdf_device(d_ll.data_ptr())

    def time_steps(eng, n, first):
        """Device time of n evaluations (graph replays, no per-kernel events), each
        bracketed by CUDA events on the engine's stream, L2 flushed before each."""
        eng.set_stream(stream.cuda_stream)
        eng.enable_timing(False)
        eng.enable_graph(True)
        for k in range(args.warmup):
            flush.zero_()
            dev_step(eng, first + k)
        eng.synchronize()
        st = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        for i in range(n):
            flush.zero_()
            st[i].record(stream)
            dev_step(eng, first + args.warmup + i)
            en[i].record(stream)
        eng.synchronize()
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in zip(st, en)]

    def phase_times(eng, n, first):
        """Per-kernel device times (the engine's own events, eager launches)."""
        eng.set_stream(stream.cuda_stream)
        eng.enable_graph(False)
        eng.enable_timing(True)
        rows = []
        for i in range(n):
            flush.zero_()
            dev_step(eng, first + i)
            eng.synchronize()
            rows.append(eng.timing())
        eng.enable_timing(False)
        return rows

    for k in range(args.warmup):
        flush.zero_()
        dev_step(e, k)
    e.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        step_ms = time_steps(e, args.steps, 0)
        wall = time.perf_counter() - wall0
    clocks = clk.summary()
    launches = e.counts()["launches"]
    ph = phase_times(e, max(3, min(args.steps, 10)), 0)
    prune_ms = [t["prune_ms"] for t in ph]
    build_ms = [t["build_p_ms"] for t in ph]
    red_ms = [t["reduce_ms"] for t in ph]
    assert min(step_ms) >= 0.9 * statistics.mean(prune_ms), "events did not bracket the step"
    ms = statistics.mean(step_ms)
    if dist is not None:
        tt = torch.tensor([ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    value = units * world / (ms / 1e3)
    # results of the timed region's last step (the phase pass reran earlier sets)
    dev_step(e, args.warmup + args.steps - 1)
    e.synchronize()
    ll32_last = d_ll.cpu().numpy().copy()
    g32_last = d_grad.cpu().numpy().copy()

    # e2e through the C ABI with host buffers
    ll_h = np.zeros(M)
    g_h = np.zeros(G)
    e.set_stream(0)
    e.enable_timing(False)
    e.enable_graph(True)      # each host-API evaluation replays one captured CUDA graph
    def host_step(k):
        e.set_all_branch_lengths(host_sets[k])
        if args.mode == "grad":
            e.logpdf_grad(ll_h, g_h)
        else:
            e.logpdf()

    for k in range(min(2, args.warmup)):
        host_step(k)
    e2e_t = []
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_step(args.warmup + i)
        e2e_t.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * statistics.mean(e2e_t)
    e2e = {"value": units * world / (e2e_ms / 1e3), "unit": UNIT, "ms_per_step": e2e_ms,
           "ms_per_step_min": 1e3 * min(e2e_t), "ms_per_step_median": 1e3 * statistics.median(e2e_t),
           "h2d_bytes_per_step": int(base.nbytes),
           "d2h_bytes_per_step": int((M + (G if args.mode == "grad" else 0)) * 8),
           "path": "mcphy_batch_set_all_branch_lengths + mcphy_batch_logpdf%s (host arrays), "
                   "evaluation replayed as a CUDA graph" % ("_grad" if args.mode == "grad" else "")}
    e.close()
    del e

    # plain FP64 GPU path on the same inputs (last step's branch lengths)
    fp64 = None
    err = None
    if not args.no_fp64:
        e64 = make_engine(insts, "f64")
        last = host_sets[args.warmup + args.steps - 1]
        e64.set_all_branch_lengths(last)
        if args.mode == "grad":
            ll64, g64 = e64.logpdf_grad()
        else:
            ll64, g64 = e64.logpdf(), None
        ms64 = statistics.mean(time_steps(e64, args.fp64_steps, 0))
        fp64 = {"value": units * world / (ms64 / 1e3), "ms_per_step": ms64,
                "speedup_fp32_over_fp64": (units / (ms / 1e3)) / (units / (ms64 / 1e3))}
        ll64 = np.atleast_1d(ll64)
        rel_tot = abs(ll32_last.sum() - ll64.sum()) / abs(ll64.sum())
        rel_inst = np.max(np.abs(ll32_last - ll64) / np.abs(ll64))
        rel_g = rel_g_raw = within = None
        if g64 is not None:
            gscale = np.zeros_like(g64)
            for i in range(M):
                s = slice(off[i], off[i + 1])
                gscale[s] = np.maximum(np.abs(g64[s]), 1e-2 * np.abs(g64[s]).max())
            rel_g = float(np.max(np.abs(g32_last - g64) / gscale))
            # per entry without a floor: |g32_i - g64_i| / |g64_i|
            raw = np.abs(g32_last - g64) / np.maximum(np.abs(g64), 1e-300)
            rel_g_raw = float(np.max(raw))
            within = float(np.mean(raw <= 1e-4))
        err = {"logl_total_rel": float(rel_tot), "logl_max_instance_rel": float(rel_inst),
               "grad_max_entry_rel": rel_g, "grad_floor": "1e-2 x max |g| of the instance",
               "grad_max_entry_rel_unfloored": rel_g_raw,
               "grad_entries_within_1e-4_unfloored": within,
               "within_1e-6": bool(rel_inst <= 1e-6)}
        e64.close()

    # the SIMT FP32 path on the same inputs, beside the tensor-core one
    simt = None
    if tc_path:
        e32 = make_engine(insts, "f32")
        e32.autotune()
        ms32 = statistics.mean(time_steps(e32, args.fp64_steps, 0))
        simt = {"value": units * world / (ms32 / 1e3), "ms_per_step": ms32,
                "speedup_tensor_over_simt": ms32 / ms}
        e32.close()

    real_b = 4
    K0 = insts[0].K
    kp = 2 if K0 <= 2 else 4 if K0 <= 4 else 8 if K0 <= 8 else 20 if K0 <= 20 else 32
    if tc_path:
        alg = tc_algorithmic_bytes(insts, args.mode == "grad", prec)
        kname = "prune_tc_kernel<%d,%s>" % ((K0 + 7) // 8 * 8, prec)
    elif sweep == "level":
        alg = level_algorithmic_bytes(insts, real_b, args.mode == "grad")
        kname = "prune_level_kernel<%d,float>" % kp
    else:
        alg = algorithmic_bytes(insts, tiles[0], real_b, args.mode == "grad")
        # the benchmark workloads' leaves are all table-row codes: the row-code walk
        # unless the general one is asked for
        kname = ("prune_kernel<%d,float,%d>" % (kp, tiles[0]) if args.walk == "general" else
                 "prune_rows_kernel<%d,float,%d%s>" % (kp, tiles[0], ",%d" % rpw if rpw > 1 else ""))
    pr = statistics.mean(prune_ms)
    achieved = alg / (pr / 1e3) / 1e9
    # DRAM bytes of one prune launch from the committed ncu capture: bytes per unit
    # of the captured workload times this launch's units (traffic grows with units)
    traffic = None
    traffic_note = None
    tpath = os.path.join(ROOT, "profiles", "prune_traffic.json")
    if os.path.exists(tpath):
        try:
            tj = json.load(open(tpath))
            tj = tj.get(kname, tj) if isinstance(tj, dict) else tj
            if tj.get("kernel") == kname and (tc_path or insts[0].K == 4):
                traffic = float(tj["bytes_per_unit"]) * units
                traffic_note = (f"ncu dram bytes of a {tj['captured_workload']} launch scaled by "
                                f"units ({tj['bytes_per_unit']} B/unit)")
        except Exception:
            traffic = None
    # the level-synchronous streaming contract (5 K b bytes per unit for logL + gradient,
    # 1.5 K b for logL only, b = 4): what a design that streams every partial would move
    contract_bpu = (5.0 if args.mode == "grad" else 1.5) * insts[0].K * 4
    contract = {"bytes_per_unit": contract_bpu,
                "achieved": contract_bpu * units / (pr / 1e3) / 1e9,
                "frac": contract_bpu * units / (pr / 1e3) / 1e9 / hbm_peak,
                "note": "bytes a level-synchronous design would stream; this kernel keeps "
                        "pre-order partials and Down vectors on chip, so its own bytes "
                        "(algorithmic_bytes_per_unit) are the roofline numerator"}
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic, "traffic_source": traffic_note,
                "kernel": kname,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": alg,
                "algorithmic_bytes_per_unit": alg / units,
                "kernel_ms": pr, "share_of_step": pr / ms, "streaming_contract": contract}

    cpu = None
    if rank == 0 and not args.no_cpu:
        ref = cpu_leg(args)
        cpu = {"value": ref["value"], "unit": UNIT, "cores": ref["cpu_baseline"]["cores"],
               "kind": "port",
               "sample": "oracle (FP64, OpenMP) in a child process: the reference arm, "
                         f"{args.cpu_steps} steps of {ref['cpu_baseline']['sample']}"}

    metric = METRIC if args.mode == "grad" else \
        "logL-only site-node updates/s, FP32-scaled vs plain FP64 GPU at ≤1e-6 rel err"
    out = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": prec,
           "data": "synthetic (seeded simulation down Yule trees)",
           "config": dict(cfg, tiles={"sites_per_thread": tiles[0], "threads_per_block": tiles[1],
                                      "rates_per_warp": rpw},
                          sweep=sweep,
                          l2="flushed between steps (512 MB write, outside the timed events)",
                          parallelism="replicas" if world > 1 else "single GPU"),
           "clocks": clocks, "e2e": e2e,
           "gpu_launches": launches * args.steps,
           "roofline": roofline, "cpu_baseline": cpu, "fp64_plain": fp64,
           "error_vs_fp64": err, "fp32_simt": simt,
           "kernel_ms": {"build_transition": statistics.mean(build_ms), "prune": pr,
                         "reduce": statistics.mean(red_ms)},
           "autotune_prune_ms": tune, "wall_s_timed_loop": wall}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched-hky-g4")
    ap.add_argument("--tiles", default="auto", help="auto or SPTxTPB, e.g. 2x256")
    ap.add_argument("--site-scale", type=float, default=1.0,
                    help="scale every instance's site count (profiling cases that fit an ncu "
                         "capture; the benchmark is 1.0)")
    ap.add_argument("--walk", default="auto", choices=["auto", "general"],
                    help="general: run the general tree-walk kernel instead of the row-code one")
    ap.add_argument("--rates-per-warp", type=int, default=0, choices=[0, 1, 2, 4],
                    help="rate categories per warp of the FP32 tree walk (0: the autotuner's)")
    ap.add_argument("--sweep", default="auto", choices=["auto", "walk", "level"],
                    help="SIMT sweep; auto with --tiles auto runs the library's autotuner")
    ap.add_argument("--mode", default="grad", choices=["grad", "logl", "nuts"],
                    help="grad: logL + gradient (the headline metric); logl: logL only; "
                         "nuts: PNUTS ESS/s on a single-tree workload")
    ap.add_argument("--nuts-iter", type=int, default=0,
                    help="sampling iterations (0: 2000 on restriction-g4-bd, else 1000)")
    ap.add_argument("--nuts-adapt", type=int, default=200)
    ap.add_argument("--nuts-seed", type=int, default=1)
    ap.add_argument("--nuts-target", type=float, default=0.8)
    ap.add_argument("--nuts-plus-forward", action="store_true",
                    help="non-parity sampler variant: the plus end of a trajectory starts "
                         "with direction +1 (the reference starts both ends with -1)")
    ap.add_argument("--precision", default="f32", choices=["f32", "tf32", "bf16", "tf32x3"],
                    help="f32: FP32-scaled SIMT path; tf32 / bf16 / tf32x3: tensor-core node "
                         "updates with TF32 / BF16 / split-TF32 operands (K >= 9)")
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="oracle time of the NUTS mode's CPU estimate")
    ap.add_argument("--cpu-steps", type=int, default=6,
                    help="timed steps of the reference arm run as the cpu_baseline leg")
    ap.add_argument("--ref-units", type=float, default=6e7,
                    help="units per step of the reference arm's bounded sample")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.mode == "nuts":
        return run_nuts(args) if rank == 0 else 0
    return run_gpu(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())
