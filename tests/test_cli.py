"""The gpsat command line: the reference's flags, verdict lines and exit
codes (reference FileManager/ParametersManager.cpp:48-61, main.cu:115-118,
Results.cu:62-155), on the reference's own CNF fixtures."""
import json
import subprocess

import pytest

from conftest import GOLDEN, ROOT

CLI = ROOT / "gpupsat_gb300" / "gpsat"


@pytest.fixture(scope="module")
def cli(gpsat):
    assert CLI.exists(), "the build makes the gpsat binary"
    return str(CLI)


def run(cli, *args, cwd=None):
    return subprocess.run([cli, *map(str, args)], capture_output=True, text=True, timeout=300, cwd=cwd)


def write_cnf(path, n_vars, clauses, header=True):
    with open(path, "w") as f:
        f.write("c written by the CLI test\n")
        if header:
            f.write(f"p cnf {n_vars} {len(clauses)}\n")
        for c in clauses:
            f.write(" ".join(map(str, c)) + " 0\n")
    return path


def test_help_version_and_bad_arguments(cli):
    r = run(cli, "--help")
    assert r.returncode == 0 and "--number-of-blocks" in r.stdout and "--sequential-as-parallel" in r.stdout
    r = run(cli, "--version")
    assert r.returncode == 0 and r.stdout.startswith("gpsat ")
    assert run(cli, "--no-such-flag").returncode == 1
    assert run(cli, "-b").returncode == 1          # missing value
    assert run(cli, "x.cnf", "-b", "0").returncode == 1


def test_missing_file_exits_255(cli, tmp_path):
    r = run(cli, tmp_path / "absent.cnf")
    assert r.returncode == 255
    assert "was not found" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("split", [("-b", 1, "-t", 1), ("-b", 2, "-t", 4), ("-p",)])
def test_reference_fixtures_through_the_cli(cli, cuda_ok, tmp_path, split):
    fixtures = json.loads((GOLDEN / "solve_golden.json").read_text())["fixtures"]
    for i, fx in enumerate(fixtures):
        path = write_cnf(tmp_path / f"f{i}.cnf", fx["n_vars"], fx["clauses"])
        r = run(cli, "-i", path, *split, "-v", 0)
        assert r.returncode == 0, r.stdout + r.stderr
        lines = r.stdout.splitlines()
        if fx["expected"] == "SAT":
            k = lines.index("SATISFIABLE")
            model = [int(x) for x in lines[k + 1].split()]
            assert model[-1] == 0 and [abs(x) for x in model[:-1]] == list(range(1, fx["n_vars"] + 1))
            assert all(any(x in set(model) for x in c) for c in fx["clauses"]), f"fixture {i}: model"
            assert lines[k + 2] == "Solution was verified"
        else:
            assert "UNSATISFIABLE" in lines, f"fixture {i}: {r.stdout}"


@pytest.mark.gpu
def test_header_mismatch_and_budget(cli, cuda_ok, tmp_path):
    # header says fewer vars and clauses than the body holds: the reference
    # warns and uses what it found
    path = tmp_path / "h.cnf"
    with open(path, "w") as f:
        f.write("p cnf 2 1\n1 2 0\n-1 3 0\n-3 -2 0\n")
    r = run(cli, path, "-b", 1, "-t", 1)
    assert r.returncode == 0
    assert "highest var found is 3" in r.stdout and "found 3 clauses" in r.stdout
    assert "SATISFIABLE" in r.stdout.splitlines()
    # a conflict budget too small for a hard instance gives UNDEFINED
    import gpupsat_gb300 as g
    lits, off = g.gen_random_ksat(77, 250, 1065, 3)
    cl = [lits[off[c]:off[c + 1]].tolist() for c in range(len(off) - 1)]
    r = run(cli, write_cnf(tmp_path / "hard.cnf", 250, cl), "-b", 1, "-t", 1, "--conflict-budget", 3)
    assert r.returncode == 0 and "UNDEFINED" in r.stdout.splitlines()
