"""GPU: the full-scan clause evaluation strategy (the reference's
BASIC_SEARCH, gpsat_bcp_set_strategy(GPSAT_BCP_FULL_SCAN)) equals the
reference's own propagate_all_clauses on its golden vectors (status, conflict
clause, implied literals in order) and the oracle's restatement on seeded
inputs, reasons and counters included, with the assignment in shared memory
and in the slot's memory."""
import numpy as np
import pytest

from conftest import compare_bcp

pytestmark = pytest.mark.gpu


def scan(gpsat, lits, off, n, tl, to, cap, **kw):
    b = gpsat.BCPBatch(gpsat.Formula(lits, off, n), impl_cap=cap, **kw)
    b.set_strategy("full_scan")
    return b.run_host(tl, to)


def test_full_scan_matches_reference_golden(gpsat, cuda_ok, scan_golden):
    for ci, c in enumerate(scan_golden):
        n = int(c["n"][0])
        g = scan(gpsat, c["lits"], c["off"], n, c["tl"], c["to"], n)
        for t in range(len(c["status"])):
            k = int(c["n_impl"][t])
            assert (g["status"][t], g["conflict"][t], g["n_impl"][t]) == (c["status"][t], c["conflict"][t], k), \
                f"case {ci} trail {t}"
            assert np.array_equal(g["impl_lit"][t, :k], c["impl_lit"][t, :k]), f"case {ci} trail {t}"


@pytest.mark.parametrize("n,ratio,k,T,lo,hi,seed", [
    (2000, 4.2, 3, 256, 0.01, 0.10, 1),
    (20000, 4.2, 3, 128, 0.01, 0.05, 2),
    (300, 21.0, 5, 128, 0.05, 0.50, 3),
    (250000, 4.2, 3, 48, 0.01, 0.03, 4),    # assignment beyond shared memory: slot memory
])
def test_full_scan_matches_oracle(gpsat, orc, cuda_ok, n, ratio, k, T, lo, hi, seed):
    m = int(round(ratio * n))
    lits, off = gpsat.gen_random_ksat(seed, n, m, k)
    tl, to = gpsat.gen_trails(seed + 40, n, T, lo, hi)
    cap = min(n, 4096)
    g = scan(gpsat, lits, off, n, tl, to, cap)
    o = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=cap, threads=8, strategy="full_scan")
    compare_bcp(g, o, label=f"full scan n={n}")
    assert np.array_equal(g["counters"], o["counters"])
    assert (g["status"] == 1).any() or n >= 250000


def test_full_scan_edge_cases_and_strategy_switch(gpsat, orc, cuda_ok):
    n = 200
    lits, off = gpsat.gen_random_ksat(8, n, 852, 3)
    trails = [[], [5], [3, -7, 3, 11], [4, 9, -4], [1, 2, 250], list(range(1, n + 1))]
    to = np.zeros(len(trails) + 1, np.int64)
    to[1:] = np.cumsum([len(t) for t in trails])
    tl = np.array([x for t in trails for x in t], np.int32)
    b = gpsat.BCPBatch(gpsat.Formula(lits, off, n), impl_cap=n)
    b.set_strategy("full_scan")
    g = b.run_host(tl, to)
    o = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=n, strategy="full_scan")
    assert list(g["status"][3:5]) == [-2, -2]
    compare_bcp(g, o, label="edge")
    # tiny implication capacity: overflow reported where the oracle reports it
    b2 = gpsat.BCPBatch(gpsat.Formula(lits, off, n), impl_cap=2)
    b2.set_strategy("full_scan")
    tl2, to2 = gpsat.gen_trails(9, n, 64, 0.05, 0.3)
    compare_bcp(b2.run_host(tl2, to2), orc.BCPOracle(lits, off, n).run(tl2, to2, impl_cap=2, strategy="full_scan"),
                label="overflow")
    # back to two watched literals on the same handle
    b.set_strategy("watched")
    compare_bcp(b.run_host(tl, to), orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=n), label="watched")
    with pytest.raises(gpsat.GpsatError):
        b.set_strategy("bogus")
