"""The C++ host interface (include/gpsat.hpp) compiled into a program the way
a user of the library would: its MaxClauseJobChooser ranks split variables as
the reference's VariableChooser does (checked against the reference's own
code, host build), and on a GPU its TrailPropagator returns the oracle's
reference-order BCP outcome."""
import subprocess

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def api_check(gpsat, tmp_path_factory):
    out = tmp_path_factory.mktemp("cpp") / "api_check"
    pkg = ROOT / "gpupsat_gb300"
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" /
                                                                                      "api_check.cpp"),
                        "-o", str(out), "-L", str(pkg), "-Wl,-rpath," + str(pkg), "-lgpsat"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def write_cnf(path, lits, off, n):
    lines = [f"p cnf {n} {len(off) - 1}"]
    for c in range(len(off) - 1):
        lines.append(" ".join(str(int(x)) for x in lits[off[c]:off[c + 1]]) + " 0")
    path.write_text("\n".join(lines) + "\n")


def ref_ranking(lits, off, n):
    import ctypes
    import platform
    from oracle.ref import build_ref
    lib = build_ref.OUT / f"libref_stock_{platform.machine()}.so"
    if not lib.exists():
        pytest.skip("host build of the reference not present")
    L = ctypes.CDLL(str(lib))
    vp = ctypes.c_void_p
    L.ref_rank_vars.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64, vp, vp]
    order = np.zeros(n, np.int32)
    score = np.zeros(n, np.int32)
    k = L.ref_rank_vars(lits.ctypes.data, off.ctypes.data, n, len(off) - 1, order.ctypes.data, score.ctypes.data)
    return order[:k], score[:k]


@pytest.mark.parametrize("seed,n,k", [(1, 60, 3), (2, 200, 5), (3, 40, 5), (4, 1000, 3)])
def test_max_clause_chooser_ranks_like_the_reference(gpsat, api_check, tmp_path, seed, n, k):
    lits, off = gpsat.gen_random_ksat(seed, n, int(round(4.2 * n)), k)
    cnf = tmp_path / "f.cnf"
    write_cnf(cnf, lits, off, n)
    depth = 12
    r = subprocess.run([str(api_check), "rank", str(cnf), str(depth)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rows = r.stdout.split("\n")
    ours = [int(x) for x in rows[0].split()]
    assert int(rows[1]) == 2 ** depth
    order, score = ref_ranking(lits, off, n)
    # the reference sorts with std::sort (ties in any order): our chosen
    # variables must carry the reference's top scores, rank by rank, and
    # where a score is unique the variable must be the same
    ev = {int(v): int(s) for v, s in zip(order, score)}
    assert [ev[v] for v in ours] == [int(s) for s in score[:depth]]
    uniq = {s for s in score[:depth] if (score == s).sum() == 1}
    for i, v in enumerate(ours):
        if int(score[i]) in uniq:
            assert v == int(order[i])


def test_solver_roles_configure_the_options(api_check):
    """The C++ roles of a default SolverConfig give the library's default
    options, except the conflict budget: a SolverConfig solves to the end
    unless given one, as the CLI does.  The reference's roles (last free
    variable, geometric restarts) set its schedule: 100 conflicts, x1.3."""
    r = subprocess.run([str(api_check), "config"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    default, parity, library = [row.split() for row in r.stdout.strip().split("\n")]
    assert default[:8] + default[9:] == library[:8] + library[9:]
    assert default[8] == "0" and int(library[8]) > 0
    decide, restart, base, factor = int(parity[0]), int(parity[1]), int(parity[2]), float(parity[3])
    assert (decide, restart, base) == (1, 2, 100) and abs(factor - 1.3) < 1e-6   # LAST_FREE, GEOMETRIC
    assert int(parity[8]) == 5000 and parity[4:8] == library[4:8]


def test_oracle_generator_matches_the_library(gpsat, orc):
    for seed, n, m, k in [(2024, 5000, 21000, 3), (5, 300, 2979, 5), (77, 60, 256, 4)]:
        a = orc.gen_random_ksat(seed, n, m, k)
        b = gpsat.gen_random_ksat(seed, n, m, k)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    for seed, n, T, lo, hi in [(7, 100000, 64, 0.01, 0.05), (3, 500, 40, 0.0, 1.0)]:
        a = orc.gen_trails(seed, n, T, lo, hi)
        b = gpsat.gen_trails(seed, n, T, lo, hi)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_device_entries_reject_a_null_trail(gpsat):
    """n_trails > 0 with no trail literals is refused before any device work."""
    import ctypes
    L = gpsat.lib()
    lits, off = gpsat.gen_random_ksat(1, 50, 200, 3)
    f = gpsat.Formula(lits, off, 50)
    bufs = [np.zeros(8, np.int64) for _ in range(8)]
    p = [b.ctypes.data for b in bufs]
    rc = L.gpsat_bcp_run_static(f.handle, 64, 0, None, p[0], 2, p[1], p[2], p[3], p[4], p[5], p[6], None, None)
    assert rc == -1
    assert "bad argument" in L.gpsat_last_error().decode()
    # the argument check comes before the handle is used, so any non-null
    # handle value reaches it
    fake = ctypes.c_void_p(bufs[7].ctypes.data)
    rc = L.gpsat_bcp_run_device(fake, None, p[0], 2, p[1], p[2], p[3], p[4], p[5], p[6], None, None)
    assert rc == -1


@pytest.mark.gpu
@pytest.mark.parametrize("strategy", ["watched", "full_scan"])
def test_trail_propagator_matches_the_oracle(gpsat, orc, api_check, cuda_ok, tmp_path, strategy):
    n, m, T = 3000, 12600, 24
    lits, off = gpsat.gen_random_ksat(31, n, m, 3)
    tl, to = gpsat.gen_trails(32, n, T, 0.01, 0.12)
    cnf = tmp_path / "f.cnf"
    write_cnf(cnf, lits, off, n)
    tr = tmp_path / "trails.txt"
    tr.write_text("".join(" ".join(str(int(x)) for x in tl[to[t]:to[t + 1]]) + " 0\n" for t in range(T)))
    extra = ["scan"] if strategy == "full_scan" else []
    r = subprocess.run([str(api_check), "trails", str(cnf), str(tr), *extra], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ref = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=4096, strategy=strategy)
    rows = r.stdout.strip().split("\n")
    assert len(rows) == T
    for t, row in enumerate(rows):
        x = [int(v) for v in row.split()]
        assert x[:4] == [ref["status"][t], ref["conflict"][t], ref["stop"][t], ref["n_impl"][t]], f"trail {t}"
        k = x[3]
        pairs = np.array(x[4:4 + 2 * k]).reshape(k, 2)
        assert np.array_equal(pairs[:, 0], ref["impl_lit"][t, :k]) and np.array_equal(pairs[:, 1],
                                                                                      ref["impl_reason"][t, :k])
