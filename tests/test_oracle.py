"""CPU: the oracle (C restatement of the reference BCP) and the library's host
preprocessing are pinned to golden vectors produced by the reference itself
(tests/golden/make_golden.py)."""
import numpy as np

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
