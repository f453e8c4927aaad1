"""CPU: the C-ABI library loads, exports every symbol include/gpsat.h declares,
and its host-side parts (validation, preprocessing, generators, errors)
behave; no kernel is launched here."""
import ctypes
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions(header):
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gpsat_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(gpsat):
    lib = ctypes.CDLL(str(gpsat.LIB_PATH))
    names = declared_functions("gpsat.h")
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_header_is_plain_c_and_links(gpsat, tmp_path):
    """include/gpsat.h compiles as ISO C99 (no C++ types at the boundary), and a
    C program that takes the address of every declared function links against
    the library and runs (it only asks the version string)."""
    import subprocess
    names = declared_functions("gpsat.h")
    src = tmp_path / "abi_c.c"
    src.write_text("#include <stdio.h>\n#include \"gpsat.h\"\n"
                   "typedef void (*fn)(void);\nstatic const fn table[] = {\n" + "".join(f"    (fn)&{n},\n" for n in names) +
                   "};\n"
                   "int main(void)\n{\n    printf(\"%s %d\\n\", gpsat_version(), (int)(sizeof table / sizeof *table));\n"
                   "    return 0;\n}\n")
    exe = tmp_path / "abi_c"
    lib = gpsat.LIB_PATH
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                        "-I", str(ROOT / "include"), str(src), "-o", str(exe), "-L", str(lib.parent),
                        "-Wl,-rpath," + str(lib.parent), "-l" + lib.stem[3:]], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert "sm_103a" in out.stdout and out.stdout.split()[-1] == str(len(names))


def test_version_and_errors(gpsat):
    assert "sm_103a" in gpsat.version()
    L = gpsat.lib()
    assert L.gpsat_error_string(-6).decode() == "size exceeds a limit"
    h = ctypes.c_void_p()
    rc = L.gpsat_formula_create(None, None, 0, 0, ctypes.byref(h))
    assert rc == -1 and not h
    assert "n_vars" in L.gpsat_last_error().decode()


def test_formula_validation(gpsat):
    with pytest.raises(gpsat.GpsatError) as e:
        gpsat.Formula(np.array([1, 5], np.int32), np.array([0, 2], np.int64), 3)
    assert e.value.code == -4
    with pytest.raises(gpsat.GpsatError) as e:
        gpsat.Formula(np.array([1, 2], np.int32), np.array([0, 2, 1], np.int64), 3)  # offsets going back
    assert e.value.code == -4
    # an empty clause is not an error: the formula is unsatisfiable
    f = gpsat.Formula(np.array([1, 2], np.int32), np.array([0, 0, 2], np.int64), 3)
    assert f.info()["verdict"] == gpsat.UNSAT


def test_batch_offsets_are_checked_before_anything_is_read(gpsat):
    """gpsat_batch_create refuses offsets that go back, or literals that are
    missing, before it reads a clause (and before it looks for a device)."""
    vp = ctypes.c_void_p
    L = gpsat.lib()

    def create(lits, coff, foff, nv):
        h = vp()
        a = [None if x is None else vp(x.ctypes.data) for x in (lits, coff, foff, nv)]
        return L.gpsat_batch_create(*a, len(nv), ctypes.byref(h)), h

    lits = np.array([1, 2, -1, 2, 1, -2], np.int32)
    nv = np.array([2, 2], np.int32)
    for coff, foff in [(np.array([0, 2, 4, 6], np.int64), np.array([0, 2, 1], np.int64)),    # formulas going back
                       (np.array([0, 4, 2, 6], np.int64), np.array([0, 2, 3], np.int64)),    # clauses going back
                       (np.array([-2, 2, 4, 6], np.int64), np.array([0, 1, 3], np.int64))]:  # negative
        rc, h = create(lits, coff, foff, nv)
        assert rc == -4 and not h, L.gpsat_last_error()
    rc, h = create(None, np.array([0, 2, 4, 6], np.int64), np.array([0, 1, 3], np.int64), nv)
    assert rc == -1 and not h
    # well-formed: past the checks (no device here, or a batch made and freed)
    rc, h = create(lits, np.array([0, 2, 4, 6], np.int64), np.array([0, 1, 3], np.int64), nv)
    assert rc in (0, -7), L.gpsat_last_error()
    if rc == 0:
        L.gpsat_batch_destroy(h)


def test_preprocessing_decides_trivial_formulas(gpsat):
    assert gpsat.Formula.from_clauses([[1, -1], [2, -2, 3]]).info()["verdict"] == gpsat.SAT
    assert gpsat.Formula.from_clauses([[1], [-1], [1, 2]]).info()["verdict"] == gpsat.UNSAT
    f = gpsat.Formula.from_clauses([[1], [-1, 2, 3], [-2, 3, 4], [2, 2, -4]])
    ex = f.export()
    assert ex["verdict"] == 0
    assert list(ex["solved"]) == [1]
    assert list(ex["lits"]) == [2, 3, -2, 3, 4, 2, -4]


def test_generators_are_seeded_and_valid(gpsat):
    a, off = gpsat.gen_random_ksat(5, 100, 400, 3)
    b, _ = gpsat.gen_random_ksat(5, 100, 400, 3)
    c, _ = gpsat.gen_random_ksat(6, 100, 400, 3)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    cl = np.abs(a.reshape(-1, 3))
    assert (cl >= 1).all() and (cl <= 100).all()
    assert all(len(set(r)) == 3 for r in cl.tolist())
    assert 0.4 < (a > 0).mean() < 0.6
    tl, to = gpsat.gen_trails(9, 1000, 50, 0.01, 0.05)
    tl2, to2 = gpsat.gen_trails(9, 1000, 50, 0.01, 0.05)
    assert np.array_equal(tl, tl2) and np.array_equal(to, to2)
    lens = np.diff(to)
    assert lens.min() >= 10 and lens.max() <= 50
    for t in range(50):
        v = np.abs(tl[to[t]:to[t + 1]])
        assert len(np.unique(v)) == len(v) and v.min() >= 1 and v.max() <= 1000


def test_planted_generator(gpsat):
    n, m, G = 4000, 16000, 40
    lits, off, planted = gpsat.gen_planted(3, n, m, 3, G, 0.9)
    lits2, _, planted2 = gpsat.gen_planted(3, n, m, 3, G, 0.9)
    assert np.array_equal(lits, lits2) and np.array_equal(planted, planted2)
    cl = lits.reshape(-1, 3)
    v = np.abs(cl)
    assert v.min() >= 1 and v.max() <= n and (np.sort(v, 1)[:, 1:] != np.sort(v, 1)[:, :-1]).all()
    # the hidden assignment satisfies every clause
    assert ((np.sign(cl) == planted[v - 1]).any(1)).all()
    assert 0.3 < (planted > 0).mean() < 0.7
    # most literals share their clause's majority community
    comm = (v - 1) * G // n
    major = np.array([np.bincount(r, minlength=G).max() for r in comm])
    assert (major >= 2).mean() > 0.9
    assert gpsat.check_model(lits, off, planted, n)
    with pytest.raises(gpsat.GpsatError):
        gpsat.gen_planted(1, 50, 10, 3, 40, 0.9)   # communities of one variable cannot hold 3


def test_host_model_checker(gpsat):
    """gpsat_check_model: true for a satisfying model, false with the first
    falsified clause otherwise; bad offsets and literals are errors."""
    lits = np.array([1, 2, -1, 3, -2, -3], np.int32)
    off = np.array([0, 2, 4, 6], np.int64)
    assert gpsat.check_model(lits, off, np.array([1, -1, 1], np.int8), 3)
    bad = ctypes.c_int64()
    m = np.array([-1, -1, 1], np.int8)
    L = gpsat.lib()
    vp = ctypes.c_void_p
    assert L.gpsat_check_model(vp(lits.ctypes.data), vp(off.ctypes.data), 3, vp(m.ctypes.data), 3,
                               ctypes.byref(bad)) == 0 and bad.value == 0
    good = np.array([1, -1, 1], np.int8)   # the scan reaches every clause
    with pytest.raises(gpsat.GpsatError):
        gpsat.check_model(lits, np.array([0, 4, 2, 6], np.int64), good, 3)    # offsets going back
    with pytest.raises(gpsat.GpsatError):
        gpsat.check_model(lits, off, good, 2)                                  # literal 3 out of range
    assert L.gpsat_check_model(None, vp(off.ctypes.data), 3, vp(m.ctypes.data), 3, None) == -1


def test_bcp_without_device_fails_loudly(gpsat):
    if gpsat.device_count() > 0:
        pytest.skip("a GPU is visible; covered by the GPU tests")
    lits, off = gpsat.gen_random_ksat(1, 50, 200, 3)
    f = gpsat.Formula(lits, off, 50)
    with pytest.raises(gpsat.GpsatError) as e:
        gpsat.BCPBatch(f, impl_cap=64)
    assert e.value.code == -7


def test_cube_jobs_follow_the_reference_chooser(gpsat):
    from gpupsat_gb300 import jobs
    # var 3 occurs 3 times (score 3*2), var 2 twice (2*1), var 1 once (0)
    lits = np.array([1, 2, 3, -2, 3, -3], np.int32)
    assert list(jobs.rank_variables(lits, 3)) == [3, 2, 1]
    assert list(jobs.rank_variables(lits, 3, "occurrences")) == [3, 2, 1]
    assert list(jobs.rank_variables(lits, 3, scores=[5.0, 1.0, 5.0])) == [1, 3, 2]
    jf, co, cl = jobs.cube_jobs([(lits, np.array([0, 3, 6]))], [3], depth=2)
    assert list(jf) == [0] * 4 and list(co) == [0, 2, 4, 6, 8]
    # depth first, positive before negative
    assert cl.reshape(4, 2).tolist() == [[3, 2], [3, -2], [-3, 2], [-3, -2]]
    jf, co, cl = jobs.cube_jobs([(lits, None), (lits, None)], [3, 3], depth=0)
    assert list(jf) == [0, 1] and list(co) == [0, 0, 0] and len(cl) == 0


def test_dimacs_parser(gpsat):
    # the reference's grammar (FileManager/CnfReader.cpp:40-47): comments, then
    # the header, then clauses terminated by 0; the highest variable found wins
    text = "c a comment\nc\n\np cnf 3 2\n1 -2 0\n2 3 -1 0\n"
    d = gpsat.parse_dimacs(text)
    assert d["n_vars"] == 3 and d["header_vars"] == 3 and d["header_clauses"] == 2
    assert list(d["lits"]) == [1, -2, 2, 3, -1] and list(d["offsets"]) == [0, 2, 5]
    # the header may undercount; several clauses on a line and a trailing % are accepted
    d = gpsat.parse_dimacs("p cnf 2 1\n1 4 0 -4 2 0\n%\n0\n")
    assert d["n_vars"] == 4 and list(d["offsets"]) == [0, 2, 4]
    # "0" alone is an empty clause: the formula is unsatisfiable
    d = gpsat.parse_dimacs("p cnf 2 2\n1 2 0\n0\n")
    assert list(d["offsets"]) == [0, 2, 2]
    f = gpsat.Formula(d["lits"], d["offsets"], 2)
    assert f.info()["verdict"] == gpsat.UNSAT
    for bad in ("1 2 0\n", "p cnf x 1\n1 0\n", "p cnf 2 1\n1 2\n", "p dnf 2 1\n1 0\n", "p cnf 2 1\n1 a 0\n"):
        with pytest.raises(gpsat.GpsatError) as e:
            gpsat.parse_dimacs(bad)
        assert e.value.code == -5, bad
