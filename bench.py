"""Benchmark: reference-order two-watched-literal BCP propagations/s on GB300.

Workload (the BCP microbenchmark configuration): seeded uniform random 3-SAT,
n = 1,000,000 variables, m = 4,200,000 clauses (int32 signed-literal CSR arena);
4096 independent seeded partial trails per step, each assigning a uniformly
random 1-5% of the variables with random polarity at decision level 1.  One
step = one pass of the BCP kernel over all 4096 trails (every trail literal
assigned, then propagated in trail order depth-first until the first
conflict, as the reference applies assumptions).  Outputs per trail: implied
literals in order, reason clauses, conflict flag / clause, stop index.

  value   propagations/s with inputs resident in HBM (CUDA events on the
          launch stream, K back-to-back launches)
  e2e     propagations/s through gpsat_bcp_run_host: pinned host trails in,
          results out, copies inside the timed region
  roofline  algorithmic bytes per launch (4*watch entries + 4*clause
          literals + 1*assignment lookups + 9*implications + 5*trail
          literals, counted by the kernel) / average launch time, against the
          measured HBM copy bandwidth
  cpu_baseline  the oracle's C restatement of the reference BCP (same
          semantics and outputs) on the host cores, on a bounded sample

Beside the BCP figures the default line carries two more measurements of the
same run (each skipped with --no-solve / --no-latency):
  solve     the batched solve workload: 16,384 seeded random 3-SAT instances,
            n ~ U[50, 250], m = round(4.26 n), one persistent launch, 10^5
            conflicts per instance; decided instances/s, verdict counts, every
            SAT model checked on the device and on the host, and the verdicts
            compared with the reference's own (recorded in tests/golden)
  latency   single-instance solving: 40 seeded n=50, m=213 instances, one
            solve call each; milliseconds per call

`--impl reference` times the reference's CPU path alone: the BCP restatement
on all host cores, its own solver (host build, iteration cap lifted, a wall
budget per instance, one process per core) on a sample of the solve
workload, its own solver per single instance on one core, and its own BCP at
a scaled-down n.  Its inputs come from the oracle's generator, so that arm
loads nothing of the shipped library.  Under torchrun each rank runs its own
4096 trails (weak scaling; trails never exchange data) and rank 0 prints one
JSON line.
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

METRIC = "BCP props/s"
UNIT = "props/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpsat", choices=["gpsat", "reference"])
    ap.add_argument("--n-vars", type=int, default=1_000_000)
    ap.add_argument("--ratio", type=float, default=4.2)
    ap.add_argument("--trails", type=int, default=4096)
    ap.add_argument("--impl-cap", type=int, default=4096)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-trails", type=int, default=4096)
    ap.add_argument("--slots", type=int, default=None,
                    help="bcp: trails in flight (default: the autotuner's choice, timed on warm-up launches)")
    ap.add_argument("--arena-cap", type=int, default=0,
                    help="bcp: added watch entries per trail slot (default: the library's, 2^17)")
    ap.add_argument("--order-pivot", type=int, default=None,
                    help="bcp: trails whose literal count is nearest this start first (default: the autotuner's "
                         "choice; 0 = shortest first)")
    ap.add_argument("--window", type=int, default=None, choices=[64, 128, 256],
                    help="bcp: watch entries per round and trail (default: the autotuner's choice); with "
                         "--slots, no tuning launch runs")
    ap.add_argument("--workload", default="bcp", choices=["bcp", "solve", "planted", "seeding", "full_scan"],
                    help="bcp: the BCP microbenchmark (default); full_scan: the same trails under the "
                         "reference's full-scan clause evaluation; solve: batched random 3-SAT solving; "
                         "planted: planted community instances split into JobChooser cubes; "
                         "seeding: learned VSIDS/phase seeding against plain solving")
    ap.add_argument("--n-range", type=int, nargs=2, default=[50, 250], help="solve: variables per instance")
    ap.add_argument("--conflict-budget", type=int, default=100000, help="solve/planted/seeding: per job")
    ap.add_argument("--phase-init", type=int, default=0, choices=[0, 1, 2],
                    help="planted: first polarity of a variable (0 false, 1 true, 2 its majority sign)")
    ap.add_argument("--train-instances", type=int, default=4096, help="seeding: training formulas")
    ap.add_argument("--epochs", type=int, default=3, help="seeding: training passes")
    ap.add_argument("--train-kind", default="random", choices=["random", "planted"], help="seeding: training set")
    ap.add_argument("--eval", nargs="+", default=["batch", "random300", "planted"],
                    choices=["batch", "random300", "planted"], help="seeding: held-out sets (first one is value)")
    ap.add_argument("--instances", type=int, default=None, help="solve: 16384, planted: 128, seeding: 1024 held-out formulas")
    ap.add_argument("--depth", default="6", help="planted: split variables per instance (cubes = 2^depth), "
                                                 "or 'auto' to autotune it on a sample")
    ap.add_argument("--cpu-instances", type=int, default=256,
                    help="reference solve sample: the first N instances of the solve workload")
    ap.add_argument("--cpu-seconds", type=float, default=60.0, help="reference solve sample: wall budget")
    ap.add_argument("--ref-budget", type=float, default=5.0,
                    help="reference solve sample: wall seconds per instance before it counts as ref-undecided")
    ap.add_argument("--ref-own-trails", type=int, default=1024,
                    help="reference arm: trails of the reference's own BCP timed at n=2000")
    ap.add_argument("--no-solve", action="store_true", help="bcp: leave out the batched-solve measurement")
    ap.add_argument("--no-latency", action="store_true", help="bcp: leave out the single-instance measurement")
    ap.add_argument("--solve-instances", type=int, default=16384, help="bcp: instances of the solve measurement")
    return ap.parse_args()


def workload(args, rank, gen=None):
    """The BCP workload; gen is the module whose generators make it (the
    library's by default; the oracle's restatement of the same streams for the
    reference arm)."""
    if gen is None:
        import gpupsat_gb300 as gen
    g = gen
    n = args.n_vars
    m = int(round(args.ratio * n))
    lits, off = g.gen_random_ksat(2024, n, m, 3)
    tl, to = g.gen_trails(7 + 1000 * rank, n, args.trails, 0.01, 0.05)
    return n, m, lits, off, tl, to


def config(args, n, m):
    formula = m * 3 * 4 + m * 4 + n * 4 + 2 * m * 32          # literals, offsets, list offsets, initial watches
    trails = args.trails * 0.03 * n * 4                         # 1-5% of n per trail, int32
    slot = n // 16 * 4 + n * 4 + m * 4 + (args.arena_cap or (1 << 17)) * 32
    big = formula + trails > 256e6
    return {"workload": "BCP microbenchmark: random 3-SAT, partial trails",
            "n_vars": n, "n_clauses": m, "n_trails": args.trails, "trail_fraction": [0.01, 0.05],
            "literal_arena": "int32 CSR",
            "l2": f"formula {formula / 1e9:.3g} GB, trails {trails / 1e9:.3g} GB, per-trail state "
                  f"{slot / 1e6:.3g} MB per slot" + ("; inputs larger than L2, no flush needed" if big else
                                                    "; the formula fits L2 (a small case)"),
            "semantics": "reference order (bit-exact reasons and conflict clause)"}


class Clocks:
    """Samples nvidia-smi during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                         timeout=5).stdout.strip()
                    if out:
                        self.rows.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        for r in self.rows:
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                 r[5:9]):
                if val.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, STREAM-style copy)"
    return 6800.0, "fallback 6.8 TB/s"


def traffic_per_launch(n, trails, window, slots, pivot):
    """DRAM bytes of one launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)
    from the committed capture of this exact workload and launch shape, else None."""
    p = ROOT / "profiles" / "bcp_traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    if (d.get("n_vars"), d.get("n_trails"), d.get("window"), d.get("slots"), d.get("order_pivot", 0)) != \
            (n, trails, window, slots, pivot):
        return None
    return d["dram_bytes_per_launch"]


def alg_bytes(cnt):
    W, L, A, I, T = (cnt[:, i].sum(dtype=np.float64) for i in range(1, 6))
    return 4 * W + 4 * L + A + 9 * I + 5 * T


def cpu_baseline(lits, off, n, tl, to, ntrails, threads, strategy="watched"):
    """The oracle on the first `ntrails` trails with `threads` host threads.
    Units: propagations (watched) or clause evaluations (full_scan)."""
    import oracle
    o = oracle.BCPOracle(lits, off, n)
    T = min(ntrails, len(to) - 1)
    sub_to = to[:T + 1].copy()
    sub_tl = tl[:sub_to[-1]]
    t0 = time.perf_counter()
    r = o.run(sub_tl, sub_to, impl_cap=4096, threads=threads, strategy=strategy)
    dt = time.perf_counter() - t0
    props = int(r["counters"][:, 1 if strategy == "full_scan" else 0].sum())
    return props / dt, props, dt, T


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    n, m, lits, off, tl, to = workload(args, 0, gen=oracle)
    threads = os.cpu_count() or 1
    vals = []
    per_step = max(64, min(args.cpu_trails, args.trails))
    for s in range(args.warmup + args.steps):
        # each step: a bounded sample of the same workload (trails rotate per step)
        b = (s * per_step) % max(1, args.trails - per_step + 1)
        sub_to = to[b:b + per_step + 1] - to[b]
        sub_tl = tl[to[b]:to[b + per_step]]
        v, props, dt, T = cpu_baseline(lits, off, n, sub_tl, sub_to, per_step, threads)
        if s >= args.warmup:
            vals.append((props, dt))
    props = sum(p for p, _ in vals)
    dt = sum(d for _, d in vals)
    value = props / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / len(vals),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic: seeded uniform random 3-SAT and seeded partial trails",
            "config": config(args, n, m),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{per_step} trails per step of the same workload; the reference's own "
                                       f"BCP cannot hold n=1e6 (100k-node watch pool, O(n) per assignment), so "
                                       f"its C restatement (oracle/bcp_ref.c, bit-exact with it) is timed"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line["cpu_baseline"]["ref_own_scaled"] = ref_own_bcp_scaled(trails=args.ref_own_trails)
    if not args.no_solve:
        line["solve"] = solve_object_ref(args)
    if not args.no_latency:
        line["latency"] = latency_object_ref()
    print(json.dumps(line))


def _ref_lib(variant):
    import ctypes
    import platform
    from oracle.ref import build_ref
    L = ctypes.CDLL(str(build_ref.OUT / f"libref_{variant}_{platform.machine()}.so"))
    vp = ctypes.c_void_p
    L.ref_solve.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64, vp]
    L.ref_solve.restype = ctypes.c_int
    L.ref_bcp_timed.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64, vp, ctypes.c_int64, ctypes.c_int64] + [vp] * 6
    L.ref_bcp_timed.restype = ctypes.c_int
    return L


def ref_own_bcp_scaled(n=2000, trails=1024):
    """The reference's own BCP (its WatchedClausesList, host build) at a
    scaled-down size of the BCP workload: n=2000, m=8400, trails of 1-5% of
    the variables, one host core, one call per trail; the time is that of the
    trail application alone (ref_driver.cpp times the assignments and the
    new_decision calls, not the watch-list set-up before them)."""
    import oracle
    try:
        L = _ref_lib("stock")
    except OSError:
        # not built yet here: build it from the reference sources or the
        # carried build-dir copy, else report why there is no figure
        try:
            from oracle.ref import build_ref
            build_ref.build()
            L = _ref_lib("stock")
        except (OSError, FileNotFoundError, subprocess.CalledProcessError) as e:
            return {"unavailable": f"the reference's host build is not available here: {e}"}
    m = int(round(4.2 * n))
    lits, off = oracle.gen_random_ksat(2024, n, m, 3)
    tl, to = oracle.gen_trails(7, n, trails, 0.01, 0.05)
    props = int(oracle.BCPOracle(lits, off, n).run(tl, to, impl_cap=n)["counters"][:, 0].sum())
    a, b = np.zeros(n, np.int32), np.zeros(n, np.int32)
    k1, c1, s1 = np.zeros(1, np.int64), np.zeros(1, np.int32), np.zeros(1, np.int32)
    sec = np.zeros(1, np.float64)
    P = lambda x: x.ctypes.data
    total = 0.0
    for t in range(trails):
        tr = np.ascontiguousarray(tl[to[t]:to[t + 1]])
        L.ref_bcp_timed(P(lits), P(off), n, m, P(tr), len(tr), n, P(a), P(b), P(k1), P(c1), P(s1), P(sec))
        total += float(sec[0])
    return {"value": props / total, "unit": UNIT, "cores": 1, "kind": "reference",
            "sample": f"n={n}, m={m}, {trails} trails of 1-5% ({props} propagations, {total:.2f} s): the "
                      f"reference's own WatchedClausesList (host build), one call per trail, trail application "
                      f"timed alone"}


def combine_ranks(dist, device, seconds, units):
    """Whole-job figures over the ranks: the slowest rank's time and the sum of
    the units every rank processed (each rank works on its own trails, so
    nothing else is exchanged).  dist = None for one process."""
    import torch
    if dist is None:
        return float(seconds), float(units)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(u)
    return float(t.item()), float(u.item())


def run_gpu(args):
    import torch
    import gpupsat_gb300 as g

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)

    n, m, lits, off, tl, to = workload(args, rank)
    T = args.trails
    cap = args.impl_cap
    f = g.Formula(lits, off, n)
    # with --slots fixed, only those slots are allocated (no tuning launches)
    b = g.BCPBatch(f, impl_cap=cap, max_slots=args.slots or 0, arena_cap=args.arena_cap)
    d_tl = torch.from_numpy(tl).to(dev)
    d_to = torch.from_numpy(to).to(dev)
    out = dict(status=torch.empty(T, dtype=torch.int32, device=dev),
               conflict=torch.empty(T, dtype=torch.int32, device=dev),
               stop=torch.empty(T, dtype=torch.int32, device=dev),
               n_impl=torch.empty(T, dtype=torch.int64, device=dev),
               impl_lit=torch.empty(T, cap, dtype=torch.int32, device=dev),
               impl_reason=torch.empty(T, cap, dtype=torch.int32, device=dev),
               counters=torch.empty(T, 6, dtype=torch.int64, device=dev))
    stream = torch.cuda.Stream(device=dev)
    if args.window is not None:
        b.set_window(args.window)
    for _ in range(args.warmup):
        b.run_device(d_tl, d_to, out, stream=stream.cuda_stream)
    stream.synchronize()
    # the autotuner: window width (watch entries per round: threads per
    # trail) and trails in flight, chosen on untimed launches (outputs do not
    # depend on them)
    if args.slots is None:
        windows = (args.window,) if args.window is not None else (128, 256, 64)
        pivots = (0.0, 0.1, 0.2, 0.3, 0.4) if args.order_pivot is None else ()
        tuning = b.tune(d_tl, d_to, out, stream.cuda_stream, windows=windows, pivots=pivots)
    else:
        b.set_active_slots(args.slots)
        tuning = None
    if args.order_pivot is not None:
        b.set_order_pivot(args.order_pivot)
    active = b.active or b.window_slots(b.window)
    cnt = out["counters"].cpu().numpy()
    props_step = int(cnt[:, 0].sum())
    bytes_step = alg_bytes(cnt)

    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for i in range(args.steps):
        b.run_device(d_tl, d_to, out, stream=stream.cuda_stream)
        evs[i + 1].record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    launch_ms = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    elapsed = sum(launch_ms) / 1000.0
    cnt2 = out["counters"].cpu().numpy()
    assert int(cnt2[:, 0].sum()) == props_step, "propagation count changed between steps"
    elapsed, props_all = combine_ranks(dist, dev, elapsed, props_step)
    value = props_all * args.steps / elapsed

    # end to end through the host entry point (pinned buffers)
    e2e = None
    if not args.no_e2e:
        p_tl = torch.from_numpy(tl).pin_memory().numpy()
        p_to = torch.from_numpy(to).pin_memory().numpy()
        tdt = {np.int32: torch.int32, np.int64: torch.int64}
        pinned = lambda shape, dt: torch.empty(shape, dtype=tdt[dt], pin_memory=True).numpy()
        h_out = b.host_outputs(T, counters=True, alloc=pinned)   # reused by every step, as a caller would
        h = b.run_host(p_tl, p_to, out=h_out)  # warm the staging buffers
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            h = b.run_host(p_tl, p_to, out=h_out)
        e2e_s = time.perf_counter() - t0
        e2e_s, _ = combine_ranks(dist, dev, e2e_s, 0)
        maxn = int(h["n_impl"].max())
        d2h = T * (4 * 3 + 8 + 8 * 6) + 2 * 4 * T * (maxn if maxn * 4 < cap * 2 else cap)
        e2e = {"value": props_all * args.steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(tl.nbytes + to.nbytes), "d2h_bytes_per_step": int(d2h)}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak, peak_src = peaks()
    avg_launch_s = elapsed / args.steps
    achieved = bytes_step / avg_launch_s / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic_per_launch(n, T, b.window, active, b.pivot), "peak_source": peak_src,
            "alg_bytes_per_launch": bytes_step, "kernel": f"gpsat::bcp::w{b.window // 32}::bcp_kernel"}
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        v, props, dt, Tc = cpu_baseline(lits, off, n, tl, to, args.cpu_trails, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"first {Tc} of the {T} trails ({props} propagations, {dt:.1f} s); oracle/bcp_ref.c, "
                         f"the reference's BCP semantics restated (bit-exact with it)"}
    check = bcp_sample_check(out, lits, off, n, tl, to, cap)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic: seeded uniform random 3-SAT and seeded partial trails",
            "config": config(args, n, m),
            "launch": {"window": b.window, "threads_per_trail": b.window, "slots": active, "order_pivot": b.pivot,
                       "tuning_ms": {f"{w}x{n}/{p}": round(v, 3) for (w, n, p), v in tuning.items()} if tuning else None},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            # trail application + (order kernels when more trails than slots) + BCP kernel
            "gpu_launches": args.steps * (5 if T > active else 2),
            "kernel": f"gpsat::bcp::w{b.window // 32}::bcp_kernel",
            "props_per_step": props_step, "conflicts_per_step": int((out["status"] == 1).sum().item()),
            "check": check}
    del out, d_tl, d_to
    b.close()
    f.close()
    torch.cuda.empty_cache()
    if not args.no_solve:
        line["solve"] = solve_object_gpu(args, args.solve_instances)
    if not args.no_latency:
        line["latency"] = latency_object_gpu(args)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def bcp_sample_check(out, lits, off, n, tl, to, cap, k=64, strategy="watched"):
    """Compares k evenly spaced trails of the last timed launch's outputs with
    the oracle, bit for bit (status, conflict clause, stop index, implied
    literals and reasons in order, counters); raises on a difference."""
    import oracle
    T = len(to) - 1
    idx = np.unique(np.linspace(0, T - 1, min(k, T)).astype(np.int64))
    sub_to = np.zeros(len(idx) + 1, np.int64)
    sub_to[1:] = np.cumsum(to[idx + 1] - to[idx])
    sub_tl = np.concatenate([tl[to[i]:to[i + 1]] for i in idx])
    ref = oracle.BCPOracle(lits, off, n).run(sub_tl, sub_to, impl_cap=cap, threads=os.cpu_count() or 1,
                                             strategy=strategy)
    got = {key: out[key].cpu().numpy()[idx] for key in ("status", "conflict", "stop", "n_impl", "counters")}
    for key in ("status", "conflict", "stop", "n_impl", "counters"):
        if not np.array_equal(got[key], ref[key]):
            raise AssertionError(f"bench check: BCP {key} differs from the oracle on the timed launch")
    il = out["impl_lit"].cpu().numpy()[idx]
    ir = out["impl_reason"].cpu().numpy()[idx]
    for j in range(len(idx)):
        kk = int(ref["n_impl"][j])
        if not (np.array_equal(il[j, :kk], ref["impl_lit"][j, :kk]) and
                np.array_equal(ir[j, :kk], ref["impl_reason"][j, :kk])):
            raise AssertionError(f"bench check: implications of trail {int(idx[j])} differ from the oracle")
    return {"trails": int(len(idx)), "bit_exact": True, "against": "oracle/bcp_ref.c",
            "units": int(ref["counters"][:, 1 if strategy == "full_scan" else 0].sum())}


# ---------------------------------------------------------------- full-scan strategy
SCAN_METRIC = "full-scan clause evaluations/s"
SCAN_UNIT = "evaluations/s"


def run_scan_gpu(args):
    """The BCP workload's trails under the reference's full-scan clause
    evaluation (BASIC_SEARCH): every trail literal assigned, then sweeps over
    all clauses in index order until a sweep adds nothing or a clause is
    false.  value = clause evaluations/s (device time, inputs in HBM)."""
    import torch
    import gpupsat_gb300 as g
    torch.cuda.set_device(0)
    dev = torch.device("cuda:0")
    n, m, lits, off, tl, to = workload(args, 0)
    T, cap = args.trails, args.impl_cap
    f = g.Formula(lits, off, n)
    b = g.BCPBatch(f, impl_cap=cap, max_slots=args.slots or 0)
    b.set_strategy("full_scan")
    d_tl, d_to = torch.from_numpy(tl).to(dev), torch.from_numpy(to).to(dev)
    out = dict(status=torch.empty(T, dtype=torch.int32, device=dev),
               conflict=torch.empty(T, dtype=torch.int32, device=dev),
               stop=torch.empty(T, dtype=torch.int32, device=dev),
               n_impl=torch.empty(T, dtype=torch.int64, device=dev),
               impl_lit=torch.empty(T, cap, dtype=torch.int32, device=dev),
               impl_reason=torch.empty(T, cap, dtype=torch.int32, device=dev),
               counters=torch.empty(T, 6, dtype=torch.int64, device=dev))
    stream = torch.cuda.Stream(device=dev)
    for _ in range(args.warmup):
        b.run_device(d_tl, d_to, out, stream=stream.cuda_stream)
    stream.synchronize()
    cnt = out["counters"].cpu().numpy()
    evals_step = int(cnt[:, 1].sum())
    bytes_step = alg_bytes(cnt)
    clocks = Clocks(0)
    torch.cuda.synchronize()
    clocks.start()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for i in range(args.steps):
        b.run_device(d_tl, d_to, out, stream=stream.cuda_stream)
        evs[i + 1].record(stream)
    stream.synchronize()
    clk = clocks.stop()
    elapsed = sum(evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)) / 1000.0
    assert int(out["counters"][:, 1].sum().item()) == evals_step, "evaluation count changed between steps"
    e2e = None
    if not args.no_e2e:
        h_out = b.host_outputs(T, counters=True)
        b.run_host(tl, to, out=h_out)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            b.run_host(tl, to, out=h_out)
        e2e_s = time.perf_counter() - t0
        maxn = int(h_out["n_impl"].max())
        d2h = T * (4 * 3 + 8 + 8 * 6) + 2 * 4 * T * min(maxn, cap)
        e2e = {"value": evals_step * args.steps / e2e_s, "unit": SCAN_UNIT,
               "h2d_bytes_per_step": int(tl.nbytes + to.nbytes), "d2h_bytes_per_step": int(d2h)}
    peak, peak_src = peaks()
    achieved = bytes_step / (elapsed / args.steps) / 1e9
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        v, units, dt, Tc = cpu_baseline(lits, off, n, tl, to, args.cpu_trails, threads, strategy="full_scan")
        cpu = {"value": v, "unit": SCAN_UNIT, "cores": threads, "kind": "port",
               "sample": f"first {Tc} of the {T} trails ({units} clause evaluations, {dt:.2f} s); oracle/bcp_ref.c "
                         f"full-scan restatement (pinned to the reference's own full-scan propagation)"}
    check = bcp_sample_check(out, lits, off, n, tl, to, cap, strategy="full_scan")
    line = {"metric": SCAN_METRIC, "value": evals_step * args.steps / elapsed, "unit": SCAN_UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * elapsed / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic: seeded uniform random 3-SAT and seeded partial trails",
            "config": dict(config(args, n, m), workload="BCP trails under the reference's full-scan clause "
                                                        "evaluation (BASIC_SEARCH)",
                           l2="formula resident in L2 up to n of about 2e6; the assignment bits in shared "
                              "memory up to n = 196,608"),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_source": peak_src, "alg_bytes_per_launch": bytes_step,
                         "kernel": "gpsat::bcp::scan_kernel"},
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": args.steps * (4 if T > 1 else 1),
            "sweeps_per_step": int(cnt[:, 0].sum()), "check": check}
    print(json.dumps(line))
    b.close()
    f.close()


def run_scan_reference(args):
    """Reference arm of the full-scan workload: the oracle's restatement on
    all host cores over the same trails (the reference's own full-scan
    propagation is host-built only at small n in the tests)."""
    import oracle
    n, m, lits, off, tl, to = workload(args, 0, gen=oracle)
    threads = os.cpu_count() or 1
    per_step = max(16, min(args.cpu_trails, args.trails))
    vals = []
    for s in range(args.warmup + args.steps):
        b = (s * per_step) % max(1, args.trails - per_step + 1)
        sub_to = to[b:b + per_step + 1] - to[b]
        sub_tl = tl[to[b]:to[b + per_step]]
        v, units, dt, T = cpu_baseline(lits, off, n, sub_tl, sub_to, per_step, threads, strategy="full_scan")
        if s >= args.warmup:
            vals.append((units, dt))
    value = sum(u for u, _ in vals) / sum(d for _, d in vals)
    print(json.dumps({"impl": "reference", "metric": SCAN_METRIC, "value": value, "unit": SCAN_UNIT,
                      "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1000 * sum(d for _, d in vals) / len(vals), "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "int32",
                      "data": "synthetic: seeded uniform random 3-SAT and seeded partial trails",
                      "config": dict(config(args, n, m), workload="BCP trails under the reference's full-scan "
                                                                  "clause evaluation (BASIC_SEARCH)",
                                     l2="host run"),
                      "cpu_baseline": {"value": value, "unit": SCAN_UNIT, "cores": threads, "kind": "port",
                                       "sample": f"{per_step} trails per step of the same workload"},
                      "e2e": {"value": value, "unit": SCAN_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


# ---------------------------------------------------------------- batched solving
SOLVE_METRIC = "instances decided/s"


def solve_instances(count, first=0, n_range=(50, 250), gen=None):
    """Seeded random 3-SAT, n ~ U[n_range], m = round(4.26 n): instance i uses
    formula seed 5000 + i; the sizes come from one seeded stream."""
    if gen is None:
        import gpupsat_gb300 as gen
    ns = np.random.default_rng(11).integers(n_range[0], n_range[1] + 1, size=first + count)[first:]
    return [(int(n), *gen.gen_random_ksat(5000 + first + i, int(n), int(round(4.26 * n)), 3))
            for i, n in enumerate(ns)]


def solve_config(args, instances=None):
    lo, hi = args.n_range
    return {"workload": f"batched solve: random 3-SAT, n ~ U[{lo},{hi}], m = round(4.26 n)",
            "instances": instances or args.instances, "conflict_budget": args.conflict_budget,
            "decisions": "VSIDS", "restarts": "Luby 400", "vsids_decay": 0.99, "clause_db": "6000 + 300",
            "l2": "per-job state > L2 (one workspace slot per resident warp); no flush needed"}


def reference_verdicts():
    """The reference's own verdicts on instances of the solve workload, as
    recorded in tests/golden/solve_golden.json: index -> 10 / 20, or -1 where
    the reference did not decide within its budget."""
    p = ROOT / "tests" / "golden" / "solve_golden.json"
    if not p.exists():
        return {}
    d = json.loads(p.read_text())
    ref = {}
    for e in d.get("batch", []):
        ref[int(e["index"])] = int(e["ref_nocap"]) if e["ref_nocap"] in (10, 20) else -1
    for e in d.get("workload", {}).get("instances", []):
        ref[int(e["index"])] = int(e["ref_nocap"]) if e["ref_nocap"] in (10, 20) else -1
    return ref


def compare_with_reference(verdicts, ref, n_range=(50, 250)):
    """Counts of agreement between our verdicts and the reference's recorded ones."""
    if tuple(n_range) != (50, 250):
        return None
    cmp_ = agree = disagree = undecided_ref = undecided_ours = 0
    bad = []
    for i, rv in ref.items():
        if i >= len(verdicts):
            continue
        if rv < 0:
            undecided_ref += 1
            continue
        v = int(verdicts[i])
        if v == 0:
            undecided_ours += 1
            continue
        cmp_ += 1
        if v == rv:
            agree += 1
        else:
            disagree += 1
            bad.append(i)
    return {"recorded": sum(1 for i in ref if i < len(verdicts)), "compared": cmp_, "agree": agree,
            "disagree": disagree, "ref_undecided": undecided_ref, "unknown_here": undecided_ours,
            "disagreeing_indices": bad[:16]}


def host_model_check(batch, out):
    """Every SAT verdict's model against the original clauses, on the host
    (gpsat_check_model), independent of the device checker."""
    import gpupsat_gb300 as g
    ok = 0
    sat = np.nonzero(out["verdict"] == 10)[0]
    for f in sat:
        lits, off = batch.formula(int(f))
        ok += g.check_model(lits, off, batch.model_of(out, int(f)), int(batch.n_vars[f]))
    return int(ok), int(len(sat))


def solve_object_gpu(args, count, steps=1):
    """The batched-solve workload on the GPU.  e2e: batch creation (host
    preprocessing, upload) + solve + results back; value: solve calls on the
    resident batch."""
    import gpupsat_gb300 as g
    inst = solve_instances(count, n_range=args.n_range)
    formulas = [(l, o) for _, l, o in inst]
    nv = [n for n, _, _ in inst]
    opts = g.solve_options(conflict_budget=args.conflict_budget)
    t0 = time.perf_counter()
    b = g.Batch(formulas, nv)
    out = b.solve(opts)
    e2e_s = time.perf_counter() - t0
    clocks = Clocks(0)
    clocks.start()
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        out = b.solve(opts)
        times.append(time.perf_counter() - t0)
    clk = clocks.stop()
    v = out["verdict"]
    decided = int((v != 0).sum())
    st = out["stats"]
    dev_ok = int((out["model_ok"][v == 10] == 1).sum())
    host_ok, nsat = host_model_check(b, out)
    if dev_ok != nsat or host_ok != nsat:
        raise AssertionError(f"solve: {nsat} SAT verdicts, {dev_ok} models verified on the device, {host_ok} on "
                             f"the host")
    match = compare_with_reference(v, reference_verdicts(), args.n_range)
    if match and match["disagree"]:
        raise AssertionError(f"solve: verdicts differ from the reference's on instances {match['disagreeing_indices']}")
    h2d = sum(l.nbytes + o.nbytes for l, o in formulas)
    d2h = int(out["verdict"].nbytes + out["model"].nbytes + out["stats"].nbytes + out["model_ok"].nbytes)
    b.close()
    cert = certify_sample(args, formulas[:256], nv[:256], out["verdict"][:256])
    return {"metric": SOLVE_METRIC, "value": decided * steps / sum(times), "unit": "instances/s",
            "unsat_certified": cert,
            "steps": steps, "warmup": 1, "ms_per_step": 1000 * sum(times) / steps,
            "config": solve_config(args, count),
            "e2e": {"value": decided / e2e_s, "unit": "instances/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": d2h},
            "verdicts": {"sat": int((v == 10).sum()), "unsat": int((v == 20).sum()), "unknown": int((v == 0).sum())},
            "models_verified": {"sat": nsat, "device": dev_ok, "host": host_ok},
            "reference_verdicts": match,
            "conflicts": {"median": float(np.median(st[:, 0])), "mean": float(st[:, 0].mean()),
                          "max": int(st[:, 0].max())},
            "conflicts_per_s": float(st[:, 0].sum()) * steps / sum(times),
            "props_per_s": float(st[:, 2].sum()) * steps / sum(times), "clocks": clk,
            "gpu_launches": 2 * steps}


def certify_sample(args, formulas, nv, verdicts):
    """UNSAT verdicts certified independently of the reference: the first
    instances solved again with the device proof log on, every UNSAT job's
    learnt clauses checked on the host by reverse unit propagation
    (gpsat_check_rup) against the original clauses; where both runs decide,
    the verdicts must equal the timed run's."""
    import gpupsat_gb300 as g
    b = g.Batch(formulas, nv)
    opts = g.solve_options(conflict_budget=args.conflict_budget)
    out = b.solve(opts, proof_words=1 << 22)
    v = out["verdict"]
    both = (v != 0) & (verdicts != 0)
    if not np.array_equal(v[both], verdicts[both]):
        raise AssertionError("certification sample: verdicts differ from the timed run")
    t0 = time.perf_counter()
    cert = b.certify_unsat(v)
    dt = time.perf_counter() - t0
    ok = sum(1 for r in cert.values() if r[0])
    if ok != int((v == 20).sum()):
        raise AssertionError(f"certification sample: {int((v == 20).sum()) - ok} UNSAT proofs rejected")
    b.close()
    return {"instances": len(nv), "unsat": int((v == 20).sum()), "rup_certified": ok,
            "same_verdict_as_timed_run": int((v == verdicts).sum()),
            "check_seconds": round(dt, 2),
            "checker": "gpsat_check_rup (host, reverse unit propagation over the device proof log)"}


def solve_object_ref(args):
    """The reference's own solver (host build, iteration cap lifted) on the
    first instances of the solve workload, one process per host core, each
    instance with a wall budget: instances not decided within it are labelled
    ref-undecided (their time counts).  value = decided instances / wall s."""
    import oracle
    from oracle.ref import pool
    inst = solve_instances(args.cpu_instances, n_range=args.n_range, gen=oracle)
    r = pool.solve_budgeted(inst, "nocap", budget_s=args.ref_budget, wall_s=args.cpu_seconds)
    v = r["verdict"]
    started = v != -2
    decided = int(((v == 10) | (v == 20)).sum())
    return {"metric": SOLVE_METRIC, "value": decided / r["wall"], "unit": "instances/s",
            "config": solve_config(args, int(started.sum())),
            "cpu_baseline": {"value": decided / r["wall"], "unit": "instances/s", "cores": r["procs"],
                             "kind": "reference",
                             "sample": f"first {int(started.sum())} instances of the workload started within "
                                       f"{args.cpu_seconds:.0f} s; the reference's own solver (host build, "
                                       f"MAX_ITERATIONS lifted), {args.ref_budget:.0f} s wall budget per instance, "
                                       f"one process per core"},
            "verdicts": {"sat": int((v == 10).sum()), "unsat": int((v == 20).sum()),
                         "ref_undecided": int((v == -1).sum()), "undef": int((v == 0).sum()),
                         "worker_died": int((v == -3).sum())},
            "wall_s": r["wall"], "median_decided_s": float(np.median(r["seconds"][(v == 10) | (v == 20)]))
            if decided else None}


def latency_instances(gen=None):
    """40 seeded uniform random 3-SAT instances, n=50, m=213 (seeds 1..40)."""
    if gen is None:
        import gpupsat_gb300 as gen
    return [(s, *gen.gen_random_ksat(s, 50, 213, 3)) for s in range(1, 41)]


def latency_object_gpu(args):
    """One solve call per instance (a batch of one formula, resident on the
    device), timed on the host around the call; e2e includes creating the
    batch (preprocessing and upload)."""
    import gpupsat_gb300 as g
    gold = {}
    p = ROOT / "tests" / "golden" / "solve_golden.json"
    if p.exists():
        gold = {e["seed"]: e["ref_nocap"] for e in json.loads(p.read_text()).get("random", [])}
    opts = g.solve_options(conflict_budget=args.conflict_budget)
    call_ms, e2e_ms, agree, nsat, ok = [], [], 0, 0, 0
    for seed, lits, off in latency_instances():
        t0 = time.perf_counter()
        b = g.Batch([(lits, off)], [50])
        out = b.solve(opts)
        e2e_ms.append(1000 * (time.perf_counter() - t0))
        for _ in range(3):
            t0 = time.perf_counter()
            out = b.solve(opts)
            call_ms.append(1000 * (time.perf_counter() - t0))
        v = int(out["verdict"][0])
        agree += gold.get(seed) == v
        if v == 10:
            nsat += 1
            ok += int(out["model_ok"][0] == 1 and g.check_model(lits, off, b.model_of(out, 0), 50))
        b.close()
    return {"metric": "single-instance solve latency", "value": float(np.median(call_ms)), "unit": "ms",
            "higher_is_better": False,
            "config": {"workload": "single instance: random 3-SAT n=50, m=213, seeds 1..40", "calls": len(call_ms)},
            "p90_ms": float(np.percentile(call_ms, 90)),
            "e2e": {"value": float(np.median(e2e_ms)), "unit": "ms", "h2d_bytes_per_step": 213 * 3 * 4 + 214 * 8,
                    "d2h_bytes_per_step": 50 + 4 + 8 * 9 + 4},
            "verdicts_match_reference": f"{agree}/{len(gold) or 40}", "models_verified": f"{ok}/{nsat}"}


def latency_object_ref():
    """The reference's own solver per instance on one host core (in-process
    calls into its host build), stock and with the iteration cap lifted."""
    import oracle
    res = {}
    for variant in ("stock", "nocap"):
        L = _ref_lib(variant)
        ms, verd = [], []
        for seed, lits, off in latency_instances(gen=oracle):
            model = np.zeros(50, np.int32)
            t0 = time.perf_counter()
            v = L.ref_solve(lits.ctypes.data, off.ctypes.data, 50, 213, model.ctypes.data)
            ms.append(1000 * (time.perf_counter() - t0))
            verd.append(int(v))
        res[variant] = {"median_ms": float(np.median(ms)), "p90_ms": float(np.percentile(ms, 90)),
                        "decided": sum(x in (10, 20) for x in verd)}
    return {"metric": "single-instance solve latency", "value": res["nocap"]["median_ms"], "unit": "ms",
            "higher_is_better": False,
            "config": {"workload": "single instance: random 3-SAT n=50, m=213, seeds 1..40", "calls": 40},
            "cpu_baseline": {"value": res["nocap"]["median_ms"], "unit": "ms", "cores": 1, "kind": "reference",
                             "sample": "the reference's own solver (host build), one call per instance, one core"},
            "variants": res}


def run_solve_reference(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    o = solve_object_ref(args)
    line = {"impl": "reference", "metric": SOLVE_METRIC, "value": o["value"], "unit": "instances/s",
            "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": 1000 * o["wall_s"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic: seeded uniform random 3-SAT", "config": solve_config(args),
            "cpu_baseline": o["cpu_baseline"], "verdicts": o["verdicts"],
            "e2e": {"value": o["value"], "unit": "instances/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def planted_instances(count, first=0):
    """Planted 3-SAT, n ~ U[2000, 20000], m = 4.0 n, 40 equal communities, 90% of
    a clause's variables from its community; instance i uses seed 9000 + i."""
    import gpupsat_gb300 as g
    ns = np.random.default_rng(13).integers(2000, 20001, size=first + count)[first:]
    out = []
    for i, n in enumerate(ns):
        lits, off, _ = g.gen_planted(9000 + first + i, int(n), 4 * int(n), 3, 40, 0.9)
        out.append((int(n), lits, off))
    return out


def run_planted_gpu(args):
    import torch
    import gpupsat_gb300 as g
    from gpupsat_gb300 import jobs
    torch.cuda.set_device(0)
    inst = planted_instances(args.instances)
    formulas = [(l, o) for _, l, o in inst]
    nv = [n for n, _, _ in inst]
    opts = g.solve_options(conflict_budget=args.conflict_budget, phase_init=args.phase_init)
    tuned = None
    if args.depth == "auto":
        depth, table = jobs.autotune_depth(formulas, nv, depths=(4, 6, 8, 10), sample=16, options=opts,
                                           log=lambda m: print(m, file=sys.stderr))
        tuned = {str(d): {"decided": t[0], "seconds": round(t[1], 3)} for d, t in table.items()}
    else:
        depth = int(args.depth)
    jf, co, cl = jobs.cube_jobs(formulas, nv, depth)
    b = g.Batch(formulas, nv)
    for _ in range(args.warmup):
        out = b.solve(opts, jobs=(jf, co, cl))
    clocks = Clocks(0)
    torch.cuda.synchronize()
    clocks.start()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out = b.solve(opts, jobs=(jf, co, cl))
        times.append(time.perf_counter() - t0)
    clk = clocks.stop()
    v = out["verdict"]
    st = out["stats"]
    decided = int((v != 0).sum())
    assert (out["model_ok"][v == 10] == 1).all(), "a SAT verdict without a verified model"
    e2e_t = []
    for _ in range(max(1, min(2, args.steps))):
        t0 = time.perf_counter()
        bb = g.Batch(formulas, nv)
        bb.solve(opts, jobs=(jf, co, cl))
        e2e_t.append(time.perf_counter() - t0)
        bb.close()
    h2d = sum(l.nbytes + o.nbytes for l, o in formulas) + jf.nbytes + co.nbytes + cl.nbytes
    d2h = int(out["verdict"].nbytes + out["model"].nbytes + out["stats"].nbytes + out["model_ok"].nbytes)
    line = {"metric": "instances decided/s", "value": decided * args.steps / sum(times), "unit": "instances/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic: seeded planted 3-SAT with 40 communities",
            "config": {"workload": "structured batch: planted community 3-SAT, n ~ U[2000,20000], m = 4.0 n",
                       "instances": args.instances, "cube_depth": depth, "depth_autotune": tuned,
                       "phase_init": args.phase_init,
                       "jobs": int(len(jf)),
                       "chooser": "MaxClauseJobChooser ranking (reference VariableChooser score)",
                       "l2": "per-job state > L2; no flush needed"},
            "cpu_baseline": None, "clocks": clk,
            "e2e": {"value": decided * len(e2e_t) / sum(e2e_t), "unit": "instances/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": 2 * args.steps,
            "verdicts": {"sat": int((v == 10).sum()), "unsat": int((v == 20).sum()), "unknown": int((v == 0).sum())},
            "conflicts_per_instance": {"median": float(np.median(st[:, 0])), "max": int(st[:, 0].max())},
            "props_per_s": float(st[:, 2].sum()) * args.steps / sum(times)}
    print(json.dumps(line))


def seeding_eval_set(name, count):
    """Held-out formulas for the learned-seeding comparison: (formulas, n_vars, communities or None)."""
    import gpupsat_gb300 as g
    from gpupsat_gb300 import learn
    if name == "random300":      # 3-SAT, n = 300, ratio 4.26
        return [g.gen_random_ksat(40000 + i, 300, 1278, 3) for i in range(count)], [300] * count, None
    if name == "batch":          # the batched-solve workload's distribution, instances it does not use
        inst = solve_instances(count, first=8192)
        return [(l, o) for _, l, o in inst], [n for n, _, _ in inst], None
    if name == "planted":        # the structured workload's distribution at n ~ U[2000, 5000]
        ns = np.random.default_rng(17).integers(2000, 5001, size=count)
        f = [g.gen_planted(70000 + i, int(n), 4 * int(n), 3, 40, 0.9)[:2] for i, n in enumerate(ns)]
        return f, [int(n) for n in ns], [learn.communities_of(int(n)) for n in ns]
    raise ValueError(name)


def seeding_compare(net, formulas, nv, comm, opts):
    """Plain and seeded solves of the same formulas; the seeded arm's time
    includes the network's inference and the seed upload."""
    import gpupsat_gb300 as g
    from gpupsat_gb300 import learn
    bp, bs = g.Batch(formulas, nv), g.Batch(formulas, nv)
    bp.solve(opts)                                   # warm-up
    t0 = time.perf_counter()
    op = bp.solve(opts)
    plain_s = time.perf_counter() - t0
    learn.predict(net, formulas, nv, communities=comm)   # warm-up
    t0 = time.perf_counter()
    score, phase = learn.predict(net, formulas, nv, communities=comm)
    bs.set_seeds(*learn.seeds_from(score, phase))
    infer_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    os_ = bs.solve(opts)
    seed_s = time.perf_counter() - t0
    vp, vs = op["verdict"], os_["verdict"]
    both = (vp != 0) & (vs != 0)
    assert (vp[both] == vs[both]).all(), "seeded and plain verdicts disagree"
    assert (op["model_ok"][vp == 10] == 1).all() and (os_["model_ok"][vs == 10] == 1).all()
    dp, ds = int((vp != 0).sum()), int((vs != 0).sum())
    return {"instances": len(nv),
            "plain": {"decided": dp, "decided_per_s": dp / plain_s, "seconds": plain_s,
                      "median_conflicts": float(np.median(op["stats"][:, 0])),
                      "mean_conflicts": float(op["stats"][:, 0].mean())},
            "seeded": {"decided": ds, "decided_per_s": ds / (infer_s + seed_s), "seconds": infer_s + seed_s,
                       "inference_ms": 1000 * infer_s, "median_conflicts": float(np.median(os_["stats"][:, 0])),
                       "mean_conflicts": float(os_["stats"][:, 0].mean())}}


def run_seeding_gpu(args):
    """Learned seeding: train the network on budgeted solves of a training set
    (random k-SAT near threshold, or planted community instances), then solve
    held-out sets plain and seeded.  value = seeded instances decided/s on the
    first evaluation set, inference included; every set's plain and seeded
    figures and the network's forward throughput ride along."""
    import torch
    import gpupsat_gb300 as g
    from gpupsat_gb300 import learn
    torch.cuda.set_device(0)
    dev = torch.device("cuda:0")
    t0 = time.perf_counter()
    data = learn.training_set(args.train_instances, seed=0, kind=args.train_kind)
    net = learn.SeedNet(dev, seed=0)
    hist, _ = learn.train(net, data, epochs=args.epochs, log=lambda m: print(m, file=sys.stderr))
    train_s = time.perf_counter() - t0
    opts = g.solve_options(conflict_budget=args.conflict_budget)
    evals = {}
    for name in args.eval:
        f, nv, comm = seeding_eval_set(name, args.instances if name != "planted" else max(8, args.instances // 8))
        evals[name] = seeding_compare(net, f, nv, comm, opts)
        print(f"{name}: {json.dumps(evals[name])}", file=sys.stderr)
    # the network's forward throughput on the first evaluation set (device time)
    f, nv, comm = seeding_eval_set(args.eval[0], args.instances)
    G = learn.Graph(f, nv, dev, comm)
    ps = learn.Pass(net, G)
    ps.forward()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    ev0.record()
    for _ in range(reps):
        ps.forward()
    ev1.record()
    torch.cuda.synchronize()
    fwd_ms = ev0.elapsed_time(ev1) / reps
    D = learn.D
    flops = 2 * G.V * D * D + learn.LAYERS * (2 * G.V * D * 3 * D + 2 * G.C * D * D + 2 * G.C * D * 2 * D)
    first = evals[args.eval[0]]
    line = {"metric": "instances decided/s (learned seeding)", "value": first["seeded"]["decided_per_s"],
            "unit": "instances/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": 1000 * first["seeded"]["seconds"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 network, int32 solver",
            "data": f"synthetic: seeded {args.train_kind} training formulas, held-out sets {args.eval}",
            "config": {"workload": "learned seeding: 3-layer 64-wide message passing, VSIDS + phase seeds",
                       "train_kind": args.train_kind, "train_instances": args.train_instances,
                       "epochs": args.epochs, "held_out": args.instances, "conflict_budget": args.conflict_budget,
                       "train_seconds": round(train_s, 1), "final_losses": [round(float(x), 4) for x in hist[-1]]},
            "evals": evals,
            "network": {"forward_ms": fwd_ms, "tflops": flops / (fwd_ms * 1e-3) / 1e12, "nodes": G.V + G.C,
                        "edges": G.E},
            "gpu_launches": None}
    print(json.dumps(line))


def run_solve_gpu(args):
    import torch
    torch.cuda.set_device(0)
    o = solve_object_gpu(args, args.instances, steps=args.steps)
    cpu = None
    if not args.no_cpu:
        cpu = solve_object_ref(args)["cpu_baseline"]
    line = {"metric": SOLVE_METRIC, "value": o["value"], "unit": "instances/s", "n_gpus": 1, "steps": args.steps,
            "warmup": 1, "ms_per_step": o["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic: seeded uniform random 3-SAT",
            "config": o["config"], "cpu_baseline": cpu, "clocks": o["clocks"], "e2e": o["e2e"],
            "gpu_launches": o["gpu_launches"],
            **{k: o[k] for k in ("verdicts", "models_verified", "reference_verdicts", "conflicts", "conflicts_per_s",
                                 "props_per_s")}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.instances is None:
        args.instances = {"planted": 128, "seeding": 1024}.get(args.workload, 16384)
    if args.workload in ("solve", "planted") and args.steps == 20:
        args.steps = 1    # one batch solve is about 20 s (planted 1,024 instances: about 50 s)
    if args.workload == "seeding":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned seeding; its "
                              "solver's timed baseline is --workload solve"}))
        else:
            run_seeding_gpu(args)
    elif args.workload == "planted":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference's host-built solver did not return "
                              "within 600 s on one n=2000 planted instance (seed 9000) on an x86 host core; "
                              "see --workload solve for its timed baseline"}))
        else:
            run_planted_gpu(args)
    elif args.workload == "solve":
        if args.impl == "reference":
            run_solve_reference(args)
        else:
            run_solve_gpu(args)
    elif args.workload == "full_scan":
        if args.impl == "reference":
            run_scan_reference(args)
        else:
            run_scan_gpu(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
