"""CPU: the oracle (C restatement of the reference BCP) and the library's host
preprocessing are pinned to golden vectors produced by the reference itself
(tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import compare_bcp


def test_oracle_bcp_matches_reference_golden(orc, bcp_golden):
    for ci, c in enumerate(bcp_golden):
        o = orc.BCPOracle(c["lits"], c["off"], int(c["n"][0]))
        cap = max(1, c["impl_lit"].shape[1])
        r = o.run(c["tl"], c["to"], impl_cap=cap)
        compare_bcp(r, c, label=f"golden case {ci}")


def test_oracle_threads_agree(orc, bcp_golden):
    c = bcp_golden[3]
    o = orc.BCPOracle(c["lits"], c["off"], int(c["n"][0]))
    r1 = o.run(c["tl"], c["to"], impl_cap=256, threads=1)
    r4 = o.run(c["tl"], c["to"], impl_cap=256, threads=4)
    compare_bcp(r1, r4, label="threads")
    assert np.array_equal(r1["counters"], r4["counters"])


def test_preprocessing_matches_reference_golden(gpsat, preprocess_golden):
    n_decided = 0
    for i, c in enumerate(preprocess_golden):
        f = gpsat.Formula(c["lits"], c["off"], int(c["nv"][0]))
        ex = f.export()
        assert ex["verdict"] == int(c["verdict"][0]), f"case {i}: preprocessing verdict"
        if ex["verdict"] != 0:
            n_decided += 1
            continue
        assert np.array_equal(ex["offsets"], c["ooff"]), f"case {i}: clause boundaries"
        assert np.array_equal(ex["lits"], c["olits"]), f"case {i}: clause literals"
        # the reference's lists do not record which watch is first: compare as sets
        mine = np.sort(np.stack([ex["watch1"], ex["watch2"]]), axis=0)
        ref = np.sort(np.stack([c["w1"], c["w2"]]), axis=0)
        assert np.array_equal(mine, ref), f"case {i}: initial watches"
    assert 0 < n_decided < len(preprocess_golden)


def test_initial_watches_oracle_and_library_agree(gpsat, orc):
    lits, off = gpsat.gen_random_ksat(11, 3000, 12600, 3)
    f = gpsat.Formula(lits, off, 3000)
    ex = f.export()
    w1, w2 = orc.BCPOracle(lits, off, 3000).initial_watches()
    assert np.array_equal(ex["watch1"], w1) and np.array_equal(ex["watch2"], w2)


def test_oracle_rejects_conflicting_trail_and_accepts_repeats(orc):
    lits = np.array([1, 2, 3, -1, -2, 3, 1, -3, 2], np.int32)
    off = np.array([0, 3, 6, 9], np.int64)
    o = orc.BCPOracle(lits, off, 3)
    r = o.run(np.array([1, -1], np.int32), np.array([0, 2], np.int64), impl_cap=8)
    assert r["status"][0] == -2
    r2 = o.run(np.array([-3, -3], np.int32), np.array([0, 2], np.int64), impl_cap=8)
    assert r2["status"][0] in (0, 1)
    assert r2["counters"][0, 0] >= 2  # the repeated literal is propagated twice


def test_oracle_full_scan_matches_reference_golden(orc, scan_golden):
    """The full-scan restatement (the reference's BASIC_SEARCH) against the
    reference's own propagate_all_clauses: status, conflict clause, implied
    literals in order."""
    for ci, c in enumerate(scan_golden):
        n = int(c["n"][0])
        r = orc.BCPOracle(c["lits"], c["off"], n).run(c["tl"], c["to"], impl_cap=n, strategy="full_scan")
        for t in range(len(c["status"])):
            k = int(c["n_impl"][t])
            assert (r["status"][t], r["conflict"][t], r["n_impl"][t]) == (c["status"][t], c["conflict"][t], k), \
                f"case {ci} trail {t}"
            assert np.array_equal(r["impl_lit"][t, :k], c["impl_lit"][t, :k]), f"case {ci} trail {t}: implied literals"
        assert (c["status"] == 1).any() and (c["status"] == 0).any()


def _check_outputs(cl, n, tl, to, r, strategy):
    """The properties the reference's own unit tests assert of its BCP
    (UnitTesting: every implication has a clause that is unit for it; a
    conflict clause is all false), on the oracle's outputs."""
    BIG = np.int64(1) << 40
    for t in range(len(to) - 1):
        tr = tl[to[t]:to[t + 1]]
        k = int(r["n_impl"][t])
        imp = r["impl_lit"][t, :k]
        sgn = np.zeros(n + 1, np.int8)
        pos = np.full(n + 1, BIG, np.int64)
        sgn[np.abs(tr)] = np.sign(tr)
        pos[np.abs(tr)] = -1
        assert (pos[np.abs(imp)] == BIG).all(), f"{strategy} trail {t}: implied an assigned variable"
        sgn[np.abs(imp)] = np.sign(imp)
        pos[np.abs(imp)] = np.arange(k)
        if k:
            rc = cl[r["impl_reason"][t, :k]]
            is_unit = rc == imp[:, None]
            assert is_unit.sum(1).min() == 1
            false_before = (sgn[np.abs(rc)] == -np.sign(rc)) & (pos[np.abs(rc)] < np.arange(k)[:, None])
            assert (false_before | is_unit).all(), f"{strategy} trail {t}: a reason clause is not unit"
        if r["status"][t] == 1:
            c = cl[r["conflict"][t]]
            assert (sgn[np.abs(c)] == -np.sign(c)).all(), f"{strategy} trail {t}: conflict clause not false"


@pytest.mark.parametrize("strategy", ["watched", "full_scan"])
def test_oracle_outputs_keep_the_reference_invariants(gpsat, orc, strategy):
    n, m, T = 3000, 12600, 128
    lits, off = gpsat.gen_random_ksat(77, n, m, 3)
    tl, to = gpsat.gen_trails(78, n, T, 0.01, 0.08)
    r = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=n, threads=4, strategy=strategy)
    assert set(np.unique(r["status"])) <= {0, 1} and (r["status"] == 1).any() and (r["status"] == 0).any()
    _check_outputs(lits.reshape(-1, 3), n, tl, to, r, strategy)


def test_oracle_implies_the_last_literal_of_a_falsified_clause(gpsat, orc):
    """The reference's WatchedClausesList test: falsify all but the last
    literal of a clause and the last one is implied (or the trail conflicts
    before the propagation reaches it)."""
    n, m = 2000, 8400
    lits, off = gpsat.gen_random_ksat(79, n, m, 3)
    cl = lits.reshape(-1, 3)
    rng = np.random.default_rng(80)
    picks = rng.choice(m, 64, replace=False)
    trails = [(-cl[c, :2]).astype(np.int32) for c in picks]
    to = np.zeros(len(trails) + 1, np.int64)
    to[1:] = np.cumsum([len(t) for t in trails])
    tl = np.concatenate(trails)
    r = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=n, threads=4)
    for j, c in enumerate(picks):
        if r["status"][j] == 1:
            continue
        k = int(r["n_impl"][j])
        assert cl[c, 2] in r["impl_lit"][j, :k], f"clause {c}: its last literal was not implied"
