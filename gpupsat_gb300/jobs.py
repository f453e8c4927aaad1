"""Cube jobs for the batch solver: the reference's JobChooser, vectorised.

A job is a formula restricted to a cube: the d chosen variables fixed to one
of their 2^d sign patterns.  Cubes are enumerated as the reference's
chooser enumerates them (JobsManager/JobChooser.cu:52-90, mirrored by
gpsat::CubeJobChooser in include/gpsat.hpp): depth first over the chosen
variables in rank order, the positive literal before the negative one, so
job j's cube sets variable i (0-based rank) negative when bit (d-1-i) of j
is set.

Variable ranking:
  "max_clause"   the reference's MaxClauseJobChooser score: the sum over
                 the variable's occurrences of its 0-based index
                 (JobsManager/VariableChooser.cu:23-40); ties in index order
                 (the reference's std::sort leaves their order unspecified);
  "occurrences"  occurrence count, ties in index order;
  scores         any per-variable float scores (e.g. the learned split
                 scores), highest first, ties in index order.
"""
from __future__ import annotations

import numpy as np


def rank_variables(lits: np.ndarray, n_vars: int, rule: str = "max_clause", scores=None) -> np.ndarray:
    """1-based variables, best first (stable: ties keep index order)."""
    v = np.abs(np.asarray(lits, np.int64))
    if scores is not None:
        s = np.asarray(scores, np.float64)
        if s.shape != (n_vars,):
            raise ValueError("scores must hold one value per variable")
    elif rule == "max_clause":
        s = np.bincount(v, weights=(v - 1).astype(np.float64), minlength=n_vars + 1)[1:]
    elif rule == "occurrences":
        s = np.bincount(v, minlength=n_vars + 1)[1:].astype(np.float64)
    else:
        raise ValueError(f"unknown ranking rule {rule!r}")
    return np.argsort(-s, kind="stable").astype(np.int32) + 1


def cube_jobs(formulas, n_vars, depth: int, rule: str = "max_clause", scores=None):
    """(job_formula int32[J], cube_offsets int64[J+1], cube_lits int32[J*d])
    for every formula split on its `depth` best variables (fewer when the
    formula has fewer variables).  `scores`: None or one array per formula."""
    if depth < 0 or depth > 20:
        raise ValueError("depth must be in [0, 20]")
    jf, cl, co = [], [], [np.zeros(1, np.int64)]
    end = 0
    for f, ((lits, _), n) in enumerate(zip(formulas, n_vars)):
        d = min(depth, int(n))
        top = rank_variables(lits, int(n), rule, None if scores is None else scores[f])[:d]
        J = 1 << d
        if d:
            bits = (np.arange(J)[:, None] >> np.arange(d - 1, -1, -1)[None, :]) & 1
            cube = np.where(bits == 1, -top[None, :], top[None, :]).astype(np.int32)
        else:
            cube = np.zeros((1, 0), np.int32)
        jf.append(np.full(J, f, np.int32))
        cl.append(cube.reshape(-1))
        co.append(end + d * np.arange(1, J + 1, dtype=np.int64))
        end += d * J
    return (np.concatenate(jf) if jf else np.zeros(0, np.int32), np.concatenate(co),
            np.concatenate(cl) if cl else np.zeros(0, np.int32))


def autotune_depth(formulas, n_vars, depths=(4, 5, 6, 7, 8, 9, 10), sample: int = 16, options=None,
                   rule: str = "max_clause", communities=None, log=None):
    """Picks the split depth: solves a seeded sample of the formulas as cube
    jobs at every candidate depth and keeps the one with the most formulas
    decided per second (ties to the smaller depth).  Returns (depth, table)
    with table[d] = (decided, seconds)."""
    import time

    from . import Batch
    rng = np.random.default_rng(0)
    pick = np.sort(rng.choice(len(formulas), size=min(sample, len(formulas)), replace=False))
    f = [formulas[i] for i in pick]
    nv = [int(n_vars[i]) for i in pick]
    b = Batch(f, nv)
    table = {}
    best, best_rate = None, -1.0
    for d in depths:
        jobs = cube_jobs(f, nv, d, rule)
        t0 = time.perf_counter()
        out = b.solve(options, jobs=jobs)
        dt = time.perf_counter() - t0
        decided = int((out["verdict"] != 0).sum())
        table[d] = (decided, dt)
        rate = decided / dt
        if log:
            log(f"depth {d}: {decided}/{len(f)} decided in {dt:.2f} s")
        if rate > best_rate:
            best, best_rate = d, rate
    return best, table
