"""GPU: verdicts on the batched-solve workload certified independently of the
reference where it cannot decide.  On the workload's first instances (n from
50 to 250, ratio 4.26): every SAT model passes the device and the host model
checkers, every UNSAT verdict's proof log (the job's learnt clauses, logged on
the device) passes the host RUP checker against the original clauses, and
every verdict the reference's own solver reached (recorded with a wall budget
per instance in tests/golden/solve_golden.json) is the same.  Cube jobs are
certified the same way, each against its cube."""
import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def workload(gpsat, count):
    ns = np.random.default_rng(11).integers(50, 251, size=16384)[:count]
    return [gpsat.gen_random_ksat(5000 + i, int(n), int(round(4.26 * n)), 3) for i, n in enumerate(ns)], \
        [int(n) for n in ns]


def reference_verdicts():
    d = json.loads((GOLDEN / "solve_golden.json").read_text())
    ref = {e["index"]: e["ref_nocap"] for e in d.get("batch", [])}
    ref.update({e["index"]: e["ref_nocap"] for e in d.get("workload", {}).get("instances", [])})
    return ref


def test_workload_verdicts_certified(gpsat, cuda_ok):
    ref = reference_verdicts()
    count = 256
    formulas, nv = workload(gpsat, count)
    assert max(nv) > 240 and min(nv) < 60
    b = gpsat.Batch(formulas, nv)
    out = b.solve(gpsat.solve_options(conflict_budget=100000), proof_words=1 << 22)
    v = out["verdict"]
    sat = np.nonzero(v == gpsat.SAT)[0]
    unsat = np.nonzero(v == gpsat.UNSAT)[0]
    assert len(sat) > 50 and len(unsat) > 50 and (v != 0).mean() > 0.9
    for f in sat:
        lits, off = formulas[f]
        assert out["model_ok"][f] == 1 and gpsat.check_model(lits, off, b.model_of(out, f), nv[f]), f
    cert = b.certify_unsat(v)
    assert set(cert) == set(int(f) for f in unsat)
    bad = {f: r for f, r in cert.items() if not r[0]}
    assert not bad, f"UNSAT proofs rejected by the RUP checker: {dict(list(bad.items())[:5])}"
    # the reference's verdicts where it decided within its budget
    decided = [(i, r) for i, r in ref.items() if i < count and r in (10, 20) and v[i] != 0]
    assert len(decided) >= 40
    diff = [(i, r, int(v[i])) for i, r in decided if r != v[i]]
    assert not diff, f"verdicts differ from the reference's: {diff[:5]}"


def test_cube_jobs_certified(gpsat, cuda_ok):
    from gpupsat_gb300 import jobs
    formulas, nv = workload(gpsat, 24)
    jf, co, cl = jobs.cube_jobs(formulas, nv, 3)
    b = gpsat.Batch(formulas, nv)
    out = b.solve(gpsat.solve_options(conflict_budget=100000), jobs=(jf, co, cl), proof_words=1 << 21)
    cert = b.certify_unsat(out["verdict"], jobs=(jf, co, cl))
    assert cert, "no refuted cube"
    bad = {j: r for j, r in cert.items() if not r[0]}
    assert not bad, f"cube proofs rejected: {dict(list(bad.items())[:5])}"
    whole = gpsat.Batch(formulas, nv).solve(gpsat.solve_options(conflict_budget=100000))["verdict"]
    both = (whole != 0) & (out["verdict"] != 0)
    assert np.array_equal(whole[both], out["verdict"][both])
    # a formula is UNSAT only when every one of its cubes is refuted, each certified
    for f in np.nonzero(out["verdict"] == gpsat.UNSAT)[0]:
        js = [j for j in range(len(jf)) if jf[j] == f]
        assert all(j in cert and cert[j][0] for j in js)


def test_proof_log_overflow_is_reported(gpsat, cuda_ok):
    formulas, nv = workload(gpsat, 8)
    b = gpsat.Batch(formulas, nv)
    out = b.solve(gpsat.solve_options(conflict_budget=100000), proof_words=64)
    for f in range(8):
        verdict, words = b.proof(f)
        assert verdict == out["verdict"][f]
        if out["stats"][f, 0] > 40:       # more learnt clauses than 64 words hold (two or more words each)
            assert words is None
