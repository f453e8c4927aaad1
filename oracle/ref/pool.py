"""ORACLE -- test infrastructure only.

Runs the reference's own solver (the host build in oracle/_ref/, entry
`ref_solve`) on many instances with one worker process per host core and a
wall-clock budget per instance.  An instance still running at its budget is
stopped (its worker process is killed by PID and replaced) and reported as
undecided by the reference ("ref-undecided"); its time still counts toward the
pool's wall time.  Used by the golden-fixture generator and by the reference
arm / CPU baseline of bench.py -- never by the shipped library.

Workers are started with the 'spawn' method, so the pool can be created after
the parent process has touched a GPU.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import platform
import time
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent.parent / "_ref"


def _worker(variant: str, conn) -> None:
    import ctypes
    L = ctypes.CDLL(str(OUT / f"libref_{variant}_{platform.machine()}.so"))
    vp = ctypes.c_void_p
    L.ref_solve.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64, vp]
    L.ref_solve.restype = ctypes.c_int
    while True:
        job = conn.recv()
        if job is None:
            return
        idx, n, lits, off = job
        lits = np.ascontiguousarray(lits, np.int32)
        off = np.ascontiguousarray(off, np.int64)
        model = np.zeros(n, np.int32)
        t0 = time.perf_counter()
        v = L.ref_solve(lits.ctypes.data, off.ctypes.data, n, len(off) - 1, model.ctypes.data)
        conn.send((idx, int(v), time.perf_counter() - t0, model))


def solve_budgeted(instances, variant: str = "nocap", budget_s: float = 10.0, procs: int | None = None,
                   wall_s: float | None = None, want_models: bool = False) -> dict:
    """instances: list of (n_vars, lits, offsets) in DIMACS CSR form.

    Returns dict(verdict=int32[N] (10 SAT, 20 UNSAT, 0 the reference's UNDEF,
    -1 ref-undecided: stopped at the budget, -2 not started before wall_s,
    -3 its worker process died),
    seconds=float64[N] (solve time; the budget for stopped ones), wall=total
    wall seconds, procs=workers, models=list (with want_models))."""
    procs = procs or os.cpu_count() or 1
    N = len(instances)
    verdict = np.full(N, -2, np.int32)
    secs = np.zeros(N, np.float64)
    models = [None] * N if want_models else None
    ctx = mp.get_context("spawn")
    workers = {}  # slot -> [process, conn, job index or None, start time]

    def start(slot):
        a, b = ctx.Pipe()
        p = ctx.Process(target=_worker, args=(variant, b), daemon=True)
        p.start()
        workers[slot] = [p, a, None, 0.0]

    for s in range(min(procs, N)):
        start(s)
    nxt = 0
    t0 = time.perf_counter()
    try:
        while True:
            now = time.perf_counter()
            stop_new = wall_s is not None and now - t0 >= wall_s
            busy = False
            for s, w in list(workers.items()):
                p, conn, job, ts = w
                if job is None and nxt < N and not stop_new:
                    n, lits, off = instances[nxt]
                    conn.send((nxt, n, lits, off))
                    w[2], w[3] = nxt, time.perf_counter()
                    nxt += 1
                    job = w[2]
                if job is None:
                    continue
                busy = True
                if conn.poll(0) or not p.is_alive():
                    try:
                        idx, v, dt, model = conn.recv()
                    except (EOFError, OSError):
                        # the worker died without an answer: the instance is
                        # undecided; a fresh worker takes the slot
                        p.join()
                        verdict[job], secs[job] = -3, time.perf_counter() - w[3]
                        start(s)
                        continue
                    verdict[idx], secs[idx] = v, dt
                    if want_models:
                        models[idx] = model
                    w[2] = None
                elif time.perf_counter() - w[3] > budget_s:
                    p.kill()  # this worker's own PID
                    p.join()
                    conn.close()
                    verdict[job], secs[job] = -1, budget_s
                    start(s)
            if not busy and (nxt >= N or stop_new):
                break
            time.sleep(0.002)
    finally:
        wall = time.perf_counter() - t0
        for p, conn, _, _ in workers.values():
            try:
                conn.send(None)
            except Exception:
                pass
        for p, conn, _, _ in workers.values():
            p.join(timeout=2)
            if p.is_alive():
                p.kill()
                p.join()
    return dict(verdict=verdict, seconds=secs, wall=wall, procs=procs, models=models)
