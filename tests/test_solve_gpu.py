"""GPU: the device CDCL solver's verdicts equal the reference's on the same
instances (the reference's CNF fixtures and seeded random 3-SAT, verdicts
recorded from the reference itself in tests/golden/solve_golden.json), and
every SAT verdict carries a model that both the device checker and the
independent host checker accept."""
import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solve_golden():
    return json.loads((GOLDEN / "solve_golden.json").read_text())


def solve_all(gpsat, formulas, n_vars, **opts):
    b = gpsat.Batch(formulas, n_vars)
    out = b.solve(gpsat.solve_options(**opts))
    for f in range(b.n_formulas):
        if out["verdict"][f] == gpsat.SAT:
            lits, off = formulas[f]
            assert out["model_ok"][f] == 1, f"formula {f}: device checker rejected the model"
            assert gpsat.check_model(lits, off, b.model_of(out, f), n_vars[f]), f"formula {f}: host checker"
        else:
            assert out["model_ok"][f] == -1
    return out


def test_reference_fixtures(gpsat, cuda_ok, solve_golden):
    fx = solve_golden["fixtures"]
    formulas = [gpsat.clauses_to_csr(f["clauses"]) for f in fx]
    out = solve_all(gpsat, formulas, [f["n_vars"] for f in fx])
    want = [gpsat.SAT if f["expected"] == "SAT" else gpsat.UNSAT for f in fx]
    assert list(out["verdict"]) == want
    assert [f["ref_verdict"] for f in fx] == want


def random_n50(gpsat, solve_golden):
    rs = solve_golden["random"]
    return rs, [gpsat.gen_random_ksat(r["seed"], r["n"], r["m"], 3) for r in rs], [r["n"] for r in rs]


@pytest.mark.parametrize("mode", ["vsids_luby", "vsids_geometric", "last_free", "no_minimize", "majority_phase"])
def test_random_n50_matches_reference(gpsat, cuda_ok, solve_golden, mode):
    rs, formulas, nv = random_n50(gpsat, solve_golden)
    opts = dict(vsids_luby={}, vsids_geometric=dict(restart=gpsat.RESTART_GEOMETRIC, restart_base=100, restart_factor=1.3),
                last_free=dict(decide=gpsat.DECIDE_LAST_FREE), no_minimize=dict(minimize=0),
                majority_phase=dict(phase_init=2))[mode]
    out = solve_all(gpsat, formulas, nv, **opts)
    ref = [r["ref_nocap"] for r in rs]
    assert list(out["verdict"]) == ref
    # where the reference's stock iteration cap decides, it agrees too
    for r, v in zip(rs, out["verdict"]):
        if r["ref_stock"] != 0:
            assert r["ref_stock"] == v


def test_cubes_agree_with_whole_formula(gpsat, cuda_ok, solve_golden):
    rs, formulas, nv = random_n50(gpsat, solve_golden)
    whole = solve_all(gpsat, formulas, nv)["verdict"]
    # every formula split on its 3 most frequent variables: 8 cubes each
    jf, co, cl = [], [0], []
    for f, (lits, off) in enumerate(formulas):
        occ = np.bincount(np.abs(lits), minlength=nv[f] + 1)
        top = np.argsort(-occ[1:], kind="stable")[:3] + 1
        for mask in range(8):
            jf.append(f)
            cl += [int(v) if (mask >> i) & 1 else -int(v) for i, v in enumerate(top)]
            co.append(len(cl))
    b = gpsat.Batch(formulas, nv)
    out = b.solve(jobs=(np.array(jf), np.array(co), np.array(cl)))
    assert np.array_equal(out["verdict"], whole)
    assert (out["model_ok"][out["verdict"] == gpsat.SAT] == 1).all()
    assert (out["stats"][:, 8] == 8).all()


def test_batch_random_3sat_sizes(gpsat, cuda_ok):
    """n in [50, 250], ratio 4.26: SAT models verified; two different search
    configurations agree on every verdict they both reach."""
    rng = np.random.default_rng(3)
    ns = rng.integers(50, 251, size=192)
    formulas = [gpsat.gen_random_ksat(1000 + i, int(n), int(round(4.26 * n)), 3) for i, n in enumerate(ns)]
    a = solve_all(gpsat, formulas, list(ns))
    b = solve_all(gpsat, formulas, list(ns), restart=gpsat.RESTART_GEOMETRIC, restart_factor=1.3, phase_init=1)
    both = (a["verdict"] != 0) & (b["verdict"] != 0)
    assert np.array_equal(a["verdict"][both], b["verdict"][both])
    assert both.mean() > 0.9       # the rest ran out of the 10^5-conflict budget
    sat = (a["verdict"] == gpsat.SAT).mean()
    assert 0.25 < sat < 0.85


def test_preprocessing_decided_and_units(gpsat, cuda_ok):
    formulas = [gpsat.clauses_to_csr(c) for c in (
        [[1, -1], [2, 3, -2]],            # everything removed: SAT
        [[1], [-1, 2], [-2]],             # unit conflict: UNSAT
        [[1], [-1, 2, 3], [-3, 4], [-2, -4], [2, 4, 5]],
        [[1, 2], [-1, 2], [1, -2], [-1, -2]],
    )]
    out = solve_all(gpsat, formulas, [3, 2, 5, 2])
    assert list(out["verdict"]) == [gpsat.SAT, gpsat.UNSAT, gpsat.SAT, gpsat.UNSAT]


def test_conflict_budget_gives_unknown(gpsat, cuda_ok):
    lits, off = gpsat.gen_random_ksat(77, 250, 1065, 3)
    b = gpsat.Batch([(lits, off)], [250])
    out = b.solve(gpsat.solve_options(conflict_budget=5))
    assert out["verdict"][0] == gpsat.UNKNOWN
    assert out["stats"][0, 7] & 4


def test_bad_jobs_and_options_are_refused(gpsat, cuda_ok):
    """Cube offsets that do not index the cube literals, and out-of-range
    options, are refused before anything runs; the batch still solves after."""
    import ctypes
    lits, off = gpsat.gen_random_ksat(78, 40, 170, 3)
    b = gpsat.Batch([(lits, off)], [40])
    jf = np.zeros(2, np.int32)
    for co, cl in [(np.array([0, 1], np.int64), np.array([1], np.int32)),          # one offset short
                   (np.array([0, 2, 1], np.int64), np.array([1, 2], np.int32)),    # going back
                   (np.array([0, 1, 3], np.int64), np.array([1, 2], np.int32))]:   # past the literals
        with pytest.raises(gpsat.GpsatError):
            b.solve(jobs=(jf, co, cl))
    # the library's own checks: offsets with no literal array, a negative offset
    vp = ctypes.c_void_p
    verdict = np.zeros(1, np.int32)
    for co, cl in [(np.array([0, 1, 2], np.int64), None), (np.array([-1, 0, 0], np.int64), np.zeros(1, np.int32))]:
        rc = gpsat.lib().gpsat_batch_solve(b._h, None, vp(jf.ctypes.data), vp(co.ctypes.data),
                                           None if cl is None else vp(cl.ctypes.data), 2, vp(verdict.ctypes.data),
                                           None, None, None, None)
        assert rc == -1
    with pytest.raises(gpsat.GpsatError):   # a refused solve leaves no jobs to read proofs of
        b.proof(0)
    for bad in (dict(phase_init=3), dict(proof_words=-1), dict(log_participation=5)):
        with pytest.raises(gpsat.GpsatError):
            b.solve(gpsat.solve_options(**bad))
    out = b.solve(jobs=(jf, np.array([0, 1, 2], np.int64), np.array([1, -1], np.int32)))
    assert out["verdict"][0] in (gpsat.SAT, gpsat.UNSAT)
    assert out["verdict"][0] != gpsat.SAT or out["model_ok"][0] == 1
    assert out["verdict"][0] == b.solve()["verdict"][0]


def test_batched_workload_sample_matches_reference(gpsat, cuda_ok, solve_golden):
    """Instances of the batched-solve workload with n <= 150 (the first 160 of
    them), against the reference's own verdicts with its iteration cap lifted."""
    rs = solve_golden["batch"]
    formulas = [gpsat.gen_random_ksat(r["seed"], r["n"], int(round(4.26 * r["n"])), 3) for r in rs]
    out = solve_all(gpsat, formulas, [r["n"] for r in rs])
    assert (out["verdict"] != 0).all()
    decided = [(r, int(v)) for r, v in zip(rs, out["verdict"]) if r["ref_nocap"] in (10, 20)]
    assert len(decided) >= 150
    bad = [(r["index"], r["ref_nocap"], v) for r, v in decided if r["ref_nocap"] != v]
    assert not bad, f"verdicts differ from the reference: {bad[:5]}"


def test_split_depth_autotuner(gpsat, cuda_ok):
    """The JobChooser depth autotuner times a sample at each candidate depth and
    returns one of them; the cube verdicts agree with the whole-formula ones."""
    from gpupsat_gb300 import jobs
    ns = [400, 500, 600, 450, 550, 350]
    formulas = [gpsat.gen_planted(500 + i, n, 4 * n, 3, 40, 0.9)[:2] for i, n in enumerate(ns)]
    opts = gpsat.solve_options(conflict_budget=20000)
    depth, table = jobs.autotune_depth(formulas, ns, depths=(2, 3, 4), sample=4, options=opts)
    assert depth in (2, 3, 4) and set(table) == {2, 3, 4}
    assert all(t[1] > 0 for t in table.values())
    whole = gpsat.Batch(formulas, ns).solve(opts)
    cubes = gpsat.Batch(formulas, ns).solve(opts, jobs=jobs.cube_jobs(formulas, ns, depth))
    both = (whole["verdict"] != 0) & (cubes["verdict"] != 0)
    assert (whole["verdict"][both] == cubes["verdict"][both]).all()
    assert (cubes["verdict"][cubes["verdict"] != 0] == gpsat.SAT).all()    # planted: satisfiable
