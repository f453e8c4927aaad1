"""CPU: the host RUP checker (gpsat_check_rup) accepts proofs that refute a
formula by unit propagation and rejects those that do not -- a clause that
does not follow, an empty log, a satisfiable formula."""
import json

import numpy as np
import pytest

from conftest import GOLDEN


def dpll_proof(clauses, n):
    """A reverse-unit-propagation proof of an unsatisfiable formula from a
    plain DPLL search: every refuted branch contributes the negation of its
    decisions, children before parents (a leaf's clause propagates to a
    conflict by itself, an inner branch's given the clauses of the two
    branches below it)."""
    proof = []

    def up(assign):
        a = dict(assign)
        while True:
            changed = False
            for c in clauses:
                if any(a.get(abs(l)) == (l > 0) for l in c):
                    continue
                free = [l for l in c if abs(l) not in a]
                if not free:
                    return None
                if len(free) == 1:
                    a[abs(free[0])] = free[0] > 0
                    changed = True
            if not changed:
                return a

    def rec(decisions):
        a = up({abs(l): l > 0 for l in decisions})
        if a is None:
            if decisions:
                proof.append([-l for l in decisions])
            return False
        v = next((x for x in range(1, n + 1) if x not in a), None)
        if v is None:
            return True
        for lit in (v, -v):
            if rec(decisions + [lit]):
                return True
        proof.append([-l for l in decisions])
        return False

    sat = rec([])
    return sat, proof


def unit_refuted(clauses):
    """Whether unit propagation alone refutes the clauses."""
    a = {}
    while True:
        changed = False
        for c in clauses:
            if any(a.get(abs(l)) == (l > 0) for l in c):
                continue
            free = [l for l in c if abs(l) not in a]
            if not free:
                return True
            if len(free) == 1:
                a[abs(free[0])] = free[0] > 0
                changed = True
        if not changed:
            return False


def flat(proof):
    w = []
    for c in proof:
        w += [len(c)] + list(c)
    return np.array(w, np.int32)


def test_rup_accepts_dpll_proofs_of_the_unsat_fixtures(gpsat):
    d = json.loads((GOLDEN / "solve_golden.json").read_text())
    fx = [f for f in d["fixtures"] if f["expected"].upper().startswith("UNSAT")]
    assert len(fx) >= 3
    for f in fx:
        lits, off = gpsat.clauses_to_csr(f["clauses"])
        sat, proof = dpll_proof(f["clauses"], f["n_vars"])
        assert not sat
        ok, step = gpsat.check_rup(lits, off, f["n_vars"], flat(proof))
        assert ok, (f["name"], step)


def test_rup_rejects_bad_proofs(gpsat):
    rng = np.random.default_rng(3)
    done = 0
    for seed in range(40):
        n = 12
        lits, off = gpsat.gen_random_ksat(seed, n, 80, 3)
        cls = lits.reshape(-1, 3).tolist()
        sat, proof = dpll_proof(cls, n)
        if sat or len(proof) < 3 or unit_refuted(cls):
            continue
        ok, _ = gpsat.check_rup(lits, off, n, flat(proof))
        assert ok
        # no log: unit propagation over the formula alone does not refute it
        ok, step = gpsat.check_rup(lits, off, n, np.zeros(0, np.int32))
        assert not ok and step == 0
        # a log whose clauses lose their last literal no longer follows
        cut = [c[:-1] for c in proof if len(c) > 1]
        ok, step = gpsat.check_rup(lits, off, n, flat(cut))
        assert not ok
        # a unit clause that does not follow, placed first
        bad = [[int(rng.choice([-1, 1])) * int(rng.integers(1, n + 1))]] + proof
        ok, step = gpsat.check_rup(lits, off, n, flat(bad))
        if not ok:
            assert step == 0
        done += 1
    assert done >= 5


def test_rup_rejects_any_proof_of_a_satisfiable_formula(gpsat):
    lits, off = gpsat.gen_random_ksat(5, 30, 60, 3)    # ratio 2: satisfiable
    sat, _ = dpll_proof(lits.reshape(-1, 3).tolist(), 30)
    assert sat
    ok, step = gpsat.check_rup(lits, off, 30, np.zeros(0, np.int32))
    assert not ok and step == 0
    # random logs (units, binaries, ternaries, the empty clause last) never refute it
    rng = np.random.default_rng(11)
    for _ in range(200):
        log = []
        for _ in range(int(rng.integers(1, 12))):
            k = int(rng.integers(1, 4))
            vs = rng.choice(30, size=k, replace=False) + 1
            log.append([int(v) * int(rng.choice([-1, 1])) for v in vs])
        log.append([])
        ok, _ = gpsat.check_rup(lits, off, 30, flat(log))
        assert not ok


def test_rup_with_assumptions(gpsat):
    # (a | b) & (a | -b): refuted under the assumption -a, not without it
    lits, off = gpsat.clauses_to_csr([[1, 2], [1, -2]])
    assert gpsat.check_rup(lits, off, 2, np.zeros(0, np.int32), assumptions=[-1])[0]
    assert not gpsat.check_rup(lits, off, 2, np.zeros(0, np.int32))[0]
    with pytest.raises(gpsat.GpsatError):
        gpsat.check_rup(lits, off, 2, np.array([2, 1, 5], np.int32))   # literal out of range
