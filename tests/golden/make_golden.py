"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run in a container that has the reference sources, named by $GPSAT_REFERENCE
(it builds the host copy of the reference with oracle/ref/build_ref.py first):

    GPSAT_REFERENCE=<reference checkout> python tests/golden/make_golden.py
    python tests/golden/make_golden.py --workload-only   # only the workload sample
    python tests/golden/make_golden.py --scan-only       # only the full-scan vectors

Outputs (committed):
  bcp_golden.npz     formulas + trails + the reference BCP's outputs
                     (status, conflict clause, stop index, implied literals and
                     reasons), from the reference's WatchedClausesList run
                     through oracle/ref/ref_driver.cpp:ref_bcp
  preprocess_golden.npz  messy formulas and the reference's preprocessed
                     clauses, preprocessing verdict and initial watch positions
  scan_golden.npz    formulas + trails + the outputs of the reference's
                     full-scan clause evaluation (BASIC_SEARCH): status,
                     conflict clause, implied literals in order
  solve_golden.json  the reference's six CNF fixtures (tests/cnf/*.cnf, with
                     their .expected verdicts) plus seeded random 3-SAT at
                     n=50 and the verdicts of the reference's sequential solver
                     (stock iteration cap and lifted cap), the reference's
                     verdicts on n <= 150 instances of the batched-solve
                     workload ("batch"), and on its first 512 instances with a
                     wall budget per instance ("workload")
Inputs are seeded; the generator is the library's own (splitmix64 streams).
"""
from __future__ import annotations

import ctypes
import json
import os
import random
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import gpupsat_gb300 as g  # noqa: E402
from oracle.ref import build_ref  # noqa: E402

OUT = Path(__file__).resolve().parent
vp = ctypes.c_void_p


def P(a):
    return a.ctypes.data


def load(variant):
    L = ctypes.CDLL(str(build_ref.build()[variant]))
    L.ref_bcp.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64, vp, ctypes.c_int64, ctypes.c_int64] + [vp] * 5
    L.ref_solve.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64, vp]
    L.ref_preprocess.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64] + [vp] * 6
    return L


def bcp_cases(ref):
    cases = []
    specs = [  # (n, m, k, seed, trails, fmin, fmax)
        (50, 213, 3, 1, 24, 0.02, 0.30),
        (200, 852, 3, 2, 24, 0.01, 0.20),
        (1000, 4200, 3, 3, 24, 0.01, 0.08),
        (2000, 8400, 3, 4, 24, 0.01, 0.10),
        (300, 2979, 5, 5, 24, 0.10, 0.60),   # 5-SAT near threshold
    ]
    for (n, m, k, seed, T, fmin, fmax) in specs:
        lits, off = g.gen_random_ksat(seed, n, m, k)
        tl, to = g.gen_trails(seed + 1000, n, T, fmin, fmax)
        cases.append(dict(n=n, lits=lits, off=off, tl=tl, to=to))
    # long clauses (10..14 literals, beyond the kernel's register fast path):
    # signs biased against a hidden assignment, trails mostly following it,
    # so long clauses do become unit and conflicting
    R = random.Random(91)
    n = 80
    hidden = [R.random() < 0.5 for _ in range(n + 1)]
    cls = []
    for _ in range(400):
        vs = R.sample(range(1, n + 1), R.randint(10, 14))
        cls.append([v if (hidden[v] == (R.random() < 0.12)) else -v for v in vs])
    lits, off = g.clauses_to_csr(cls)
    tls, tos = [], [0]
    for t in range(24):
        vs = R.sample(range(1, n + 1), R.randint(40, 76))
        tls += [v if (hidden[v] != (R.random() < 0.04)) else -v for v in vs]
        tos.append(len(tls))
    cases.append(dict(n=n, lits=lits, off=off, tl=np.array(tls, np.int32), to=np.array(tos, np.int64)))
    # mixed-length clauses (2..9 literals, distinct variables)
    R = random.Random(77)
    n = 120
    cls = []
    for _ in range(500):
        k = R.choice([2, 2, 3, 3, 3, 4, 6, 9])
        vs = R.sample(range(1, n + 1), k)
        cls.append([v if R.random() < 0.5 else -v for v in vs])
    lits, off = g.clauses_to_csr(cls)
    tl, to = g.gen_trails(4242, n, 24, 0.02, 0.4)
    cases.append(dict(n=n, lits=lits, off=off, tl=tl, to=to))
    arrays = {}
    for ci, c in enumerate(cases):
        n, lits, off, tl, to = c["n"], c["lits"], c["off"], c["tl"], c["to"]
        T = len(to) - 1
        cap = n
        st = np.zeros(T, np.int32)
        cc = np.zeros(T, np.int32)
        si = np.zeros(T, np.int32)
        ni = np.zeros(T, np.int64)
        il = np.zeros((T, cap), np.int32)
        ir = np.zeros((T, cap), np.int32)
        for t in range(T):
            tr = np.ascontiguousarray(tl[to[t]:to[t + 1]])
            a = np.zeros(cap, np.int32)
            b = np.zeros(cap, np.int32)
            k1 = np.zeros(1, np.int64)
            c1 = np.zeros(1, np.int32)
            s1 = np.zeros(1, np.int32)
            st[t] = ref.ref_bcp(P(lits), P(off), n, len(off) - 1, P(tr), len(tr), cap, P(a), P(b), P(k1), P(c1),
                                P(s1))
            cc[t], si[t], ni[t] = c1[0], s1[0], k1[0]
            il[t], ir[t] = a, b
        kmax = max(1, int(ni.max()))
        for key, val in dict(n=np.array([n]), lits=lits, off=off, tl=tl, to=to, status=st, conflict=cc, stop=si,
                             n_impl=ni, impl_lit=il[:, :kmax], impl_reason=ir[:, :kmax]).items():
            arrays[f"c{ci}_{key}"] = val
        print(f"bcp case {ci}: n={n} statuses={np.bincount(st + 2, minlength=4)[2:]} max_impl={ni.max()}")
    arrays["n_cases"] = np.array([len(cases)])
    np.savez_compressed(OUT / "bcp_golden.npz", **arrays)


def preprocess_cases(ref):
    arrays = {}
    R = random.Random(2024)
    N = 120
    for i in range(N):
        n = R.randint(3, 25)
        m = R.randint(1, 60)
        cls = [[R.choice([-1, 1]) * R.randint(1, n) for _ in range(R.choice([1, 1, 2, 3, 3, 4, 5]))] for _ in range(m)]
        lits, off = g.clauses_to_csr(cls)
        nv = int(np.abs(lits).max())
        ol = np.zeros(len(lits) + 1, np.int32)
        oo = np.zeros(m + 2, np.int64)
        on = np.zeros(1, np.int64)
        w1 = np.zeros(m + 1, np.int32)
        w2 = np.zeros(m + 1, np.int32)
        vd = np.zeros(1, np.int32)
        ref.ref_preprocess(P(lits), P(off), nv, m, P(ol), P(oo), P(on), P(w1), P(w2), P(vd))
        k = int(on[0])
        arrays.update({f"p{i}_lits": lits, f"p{i}_off": off, f"p{i}_nv": np.array([nv]), f"p{i}_verdict": vd,
                       f"p{i}_olits": ol[:oo[k]], f"p{i}_ooff": oo[:k + 1], f"p{i}_w1": w1[:k], f"p{i}_w2": w2[:k]})
    arrays["n_cases"] = np.array([N])
    np.savez_compressed(OUT / "preprocess_golden.npz", **arrays)


def parse_dimacs(text):
    cls, cur = [], []
    for line in text.splitlines():
        line = line.strip()
        if not line or line[0] in "cp%":
            continue
        for tok in line.split():
            x = int(tok)
            if x == 0:
                cls.append(cur)
                cur = []
            else:
                cur.append(x)
    return cls


def solve_cases(stock, nocap):
    out = {"fixtures": [], "random": []}
    fx = build_ref.reference_src().parent / "tests" / "cnf"
    for cnf in sorted(fx.glob("*.cnf")):
        cls = parse_dimacs(cnf.read_text())
        lits, off = g.clauses_to_csr(cls)
        nv = int(np.abs(lits).max())
        model = np.zeros(nv, np.int32)
        v = stock.ref_solve(P(lits), P(off), nv, len(cls), P(model))
        exp = (fx / (cnf.stem + ".expected")).read_text().strip()
        out["fixtures"].append(dict(name=cnf.stem, clauses=cls, n_vars=nv, expected=exp, ref_verdict=int(v)))
    for seed in range(1, 41):
        lits, off = g.gen_random_ksat(seed, 50, 213, 3)
        model = np.zeros(50, np.int32)
        v1 = stock.ref_solve(P(lits), P(off), 50, 213, P(model))
        v2 = nocap.ref_solve(P(lits), P(off), 50, 213, P(model))
        out["random"].append(dict(seed=seed, n=50, m=213, ref_stock=int(v1), ref_nocap=int(v2)))
    (OUT / "solve_golden.json").write_text(json.dumps(out, indent=1))
    print("fixtures:", [(f["name"], f["expected"], f["ref_verdict"]) for f in out["fixtures"]])
    print("random n=50 verdicts (nocap):", [r["ref_nocap"] for r in out["random"]])


def _nocap_one(args):
    n, seed = args
    L = load("nocap")
    lits, off = g.gen_random_ksat(seed, n, int(round(4.26 * n)), 3)
    model = np.zeros(n, np.int32)
    return int(L.ref_solve(P(lits), P(off), n, len(off) - 1, P(model)))


def batch_cases():
    """The reference's verdicts (iteration cap lifted) on the batched-solve
    workload's instances with n <= 150: instance i of that workload has
    n = default_rng(11).integers(50, 251, 4096)[i] and formula seed 5000 + i."""
    import multiprocessing as mp
    ns = np.random.default_rng(11).integers(50, 251, size=4096)
    pick = [(int(ns[i]), 5000 + i, i) for i in range(4096) if ns[i] <= 150][:160]
    out = []
    with mp.get_context("spawn").Pool(os.cpu_count() or 4) as pool:
        res = [pool.apply_async(_nocap_one, ((n, seed),)) for n, seed, _ in pick]
        for (n, seed, i), r in zip(pick, res):
            try:
                v = r.get(timeout=120)
            except mp.TimeoutError:
                v = None
            out.append(dict(index=i, seed=seed, n=n, ref_nocap=v))
    data = json.loads((OUT / "solve_golden.json").read_text())
    data["batch"] = out
    (OUT / "solve_golden.json").write_text(json.dumps(data, indent=1))
    print("batch sample:", len(out), "decided by the reference:", sum(o["ref_nocap"] in (10, 20) for o in out))


def scan_cases(ref):
    """The reference's full-scan clause evaluation (ConflictAnalyzer::
    propagate_all_clauses, driven through oracle/ref/ref_driver.cpp:ref_scan)
    over seeded trails: status, conflict clause and the implied literals in
    the order the sweeps found them."""
    ref.ref_scan.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64, vp, ctypes.c_int64, ctypes.c_int64, vp, vp, vp]
    specs = [(60, 256, 3, 31, 24, 0.05, 0.25), (200, 852, 3, 32, 24, 0.02, 0.15), (1000, 4200, 3, 33, 24, 0.01, 0.06),
             (150, 1490, 5, 34, 24, 0.10, 0.50), (120, 700, 4, 35, 24, 0.05, 0.30)]
    arrays = {}
    for ci, (n, m, k, seed, T, lo, hi) in enumerate(specs):
        lits, off = g.gen_random_ksat(seed, n, m, k)
        tl, to = g.gen_trails(seed + 1000, n, T, lo, hi)
        st = np.zeros(T, np.int32)
        cc = np.zeros(T, np.int32)
        ni = np.zeros(T, np.int64)
        il = np.zeros((T, n), np.int32)
        for t in range(T):
            tr = np.ascontiguousarray(tl[to[t]:to[t + 1]])
            a = np.zeros(n, np.int32)
            k1 = np.zeros(1, np.int64)
            c1 = np.zeros(1, np.int32)
            st[t] = ref.ref_scan(P(lits), P(off), n, m, P(tr), len(tr), n, P(a), P(k1), P(c1))
            cc[t], ni[t], il[t] = c1[0], k1[0], a
        kmax = max(1, int(ni.max()))
        for key, val in dict(n=np.array([n]), lits=lits, off=off, tl=tl, to=to, status=st, conflict=cc, n_impl=ni,
                             impl_lit=il[:, :kmax]).items():
            arrays[f"c{ci}_{key}"] = val
        print(f"scan case {ci}: n={n} k={k} statuses={np.bincount(st + 2, minlength=4)[2:]} max_impl={ni.max()}")
    arrays["n_cases"] = np.array([len(specs)])
    np.savez_compressed(OUT / "scan_golden.npz", **arrays)


def workload_cases(count=512, budget_s=30.0):
    """The reference's verdicts (iteration cap lifted) on the first `count`
    instances of the batched-solve workload (n ~ U[50, 250], ratio 4.26:
    instance i has n = default_rng(11).integers(50, 251, 16384)[i] and formula
    seed 5000 + i), each with a wall budget of budget_s seconds on one host
    core; an instance not decided within it is recorded as ref-undecided (-1)."""
    from oracle.ref import pool
    ns = np.random.default_rng(11).integers(50, 251, size=16384)[:count]
    inst = []
    for i, n in enumerate(ns):
        lits, off = g.gen_random_ksat(5000 + i, int(n), int(round(4.26 * n)), 3)
        inst.append((int(n), lits, off))
    r = pool.solve_budgeted(inst, "nocap", budget_s=budget_s)
    out = [dict(index=i, seed=5000 + i, n=int(ns[i]), ref_nocap=int(r["verdict"][i]),
                seconds=round(float(r["seconds"][i]), 3)) for i in range(count)]
    data = json.loads((OUT / "solve_golden.json").read_text())
    data["workload"] = dict(budget_s=budget_s, procs=r["procs"], instances=out)
    (OUT / "solve_golden.json").write_text(json.dumps(data, indent=1))
    dec = sum(o["ref_nocap"] in (10, 20) for o in out)
    print(f"workload sample: {count} instances, {dec} decided by the reference within {budget_s} s each")


if __name__ == "__main__":
    if "--workload-only" in sys.argv:
        workload_cases()
        sys.exit(0)
    if "--scan-only" in sys.argv:
        scan_cases(load("stock"))
        sys.exit(0)
    stock, nocap = load("stock"), load("nocap")
    bcp_cases(stock)
    preprocess_cases(stock)
    solve_cases(stock, nocap)
    batch_cases()
    scan_cases(stock)
    workload_cases()
