"""ORACLE recipe -- compiles the reference's own solver sources for the host.

Test infrastructure only.  Output goes to oracle/_ref/ (git-ignored):

  oracle/_ref/src_<variant>/   build-dir copy of the reference's src/ tree
  oracle/_ref/obj_<variant>_<arch>/   objects
  oracle/_ref/libref_<variant>_<arch>.so
      stock  -- Configs.cuh as shipped (MAX_ITERATIONS 1000)
      nocap  -- MAX_ITERATIONS raised to 2e9 in the copy, nothing else changed

Recipe (nothing in the reference tree is modified):
  1. copy <reference>/src to the build dir; in the copy, replace the two
     debug print-kernel launches the host compiler cannot parse
     (SATSolver/SolverTypes.cu `print_clause_kernel <<< 1, 1>>>(c);` -> a
     direct call, Utils/CUDAClauseVec.cu `print_dev <<< 1, 1>>>(*this);` ->
     removed);
  2. compile the solver translation units with g++ and the host shim in
     oracle/ref/shim (`-include cuda_shim_pre.h`), -DNDEBUG, and
     -D__CUDA_ARCH__ everywhere except the host-side FormulaData, CUDAClauseVec
     and Preprocessing units (the device branches are the implemented ones);
  3. link them with oracle/ref/ref_driver.cpp into a shared library.

The reference checkout is named by $GPSAT_REFERENCE (the directory that holds
its src/), else CHECKOUT below.  Without either (on a machine with no
reference checkout), an existing build-dir copy under oracle/_ref/ is
compiled instead; with none of them, build() raises FileNotFoundError saying
so.
It needs Boost for nothing: the CLI/parser units that use Boost are skipped.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
SHIM = HERE / "shim"
DRIVER = HERE / "ref_driver.cpp"

# solver translation units (paths inside src/)
UNITS = [
    "BCPStrategy/ClauseListStructure.cu", "BCPStrategy/WatchedClausesList.cu",
    "ClauseLearning/LearntClauseRepository.cu", "ClauseLearning/LearntClausesManager.cu",
    "ConflictAnalysis/CUDAListGraph.cu", "ConflictAnalysis/ConflictAnalyzer.cu",
    "ConflictAnalysis/ConflictAnalyzerFullSearchSpace.cu", "ConflictAnalysis/ConflictAnalyzerWithWatchedLits.cu",
    "ConflictAnalysis/GraphAnalyzer.cu", "ConflictAnalysis/GraphStructure.cu",
    "DecisionStrategy/VSIDS.cu", "ErrorHandler/CudaMemoryErrorHandler.cu", "FileManager/FormulaData.cu",
    "Preprocessing/RepeatedLiteralsRemover.cu", "Preprocessing/UnaryClausesRemover.cu",
    "Restarts/GeometricRestartsManager.cu", "SATSolver/Backtracker.cu", "SATSolver/DecisionMaker.cu",
    "SATSolver/SATSolver.cu", "SATSolver/SolverTypes.cu", "SATSolver/VariablesStateHandler.cu",
    "Statistics/RuntimeStatistics.cu", "Utils/CUDAClauseVec.cu", "JobsManager/VariableChooser.cu",
]
HOST_SIDE = {"Utils/CUDAClauseVec.cu", "FileManager/FormulaData.cu", "Preprocessing/RepeatedLiteralsRemover.cu",
             "Preprocessing/UnaryClausesRemover.cu", "JobsManager/VariableChooser.cu"}
VARIANTS = {"stock": None, "nocap": ("#define MAX_ITERATIONS 1000", "#define MAX_ITERATIONS 2000000000")}


# where this recipe reads the reference's sources when $GPSAT_REFERENCE is not
# set: the read-only checkout of the container the library is developed in
# (absent elsewhere, where the build-dir copy under oracle/_ref/ is used)
CHECKOUT = Path("/root/reference")


def reference_src() -> Path | None:
    """src/ of the checkout named by $GPSAT_REFERENCE, else of CHECKOUT when
    it is there, else None."""
    root = os.environ.get("GPSAT_REFERENCE")
    cand = Path(root) / "src" if root else CHECKOUT / "src"
    return cand if (cand / "SATSolver" / "SATSolver.cu").exists() else None


def _patch(path: Path, old: str, new: str) -> None:
    s = path.read_text()
    if old not in s:
        raise RuntimeError(f"expected text not found in {path}: {old!r}")
    path.write_text(s.replace(old, new))


def _prepare_copy(variant: str) -> Path:
    dst = OUT / f"src_{variant}"
    ref = reference_src()
    if ref is None:
        if not (dst / "SATSolver" / "SATSolver.cu").exists():
            raise FileNotFoundError("no build-dir copy of the reference under oracle/_ref, and no reference "
                                    f"checkout at $GPSAT_REFERENCE or {CHECKOUT} (the directory holding src/)")
        return dst
    stamp = dst / ".copied"
    if stamp.exists():
        return dst
    if dst.exists():
        shutil.rmtree(dst)
    shutil.copytree(ref, dst)
    _patch(dst / "SATSolver" / "SolverTypes.cu", "print_clause_kernel <<< 1, 1>>>(c);", "print_clause(c);")
    _patch(dst / "Utils" / "CUDAClauseVec.cu", "print_dev <<< 1, 1>>>(*this);", "")
    if VARIANTS[variant]:
        _patch(dst / "SATSolver" / "Configs.cuh", *VARIANTS[variant])
    stamp.write_text("ok\n")
    return dst


def _compile(args):
    cmd, out = args
    if out.exists():
        return
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout[-4000:] + r.stderr[-4000:])


def build_variant(variant: str) -> Path:
    lib = OUT / f"libref_{variant}_{platform.machine()}.so"
    if lib.exists() and lib.stat().st_mtime >= DRIVER.stat().st_mtime:
        return lib
    src = _prepare_copy(variant)
    obj = OUT / f"obj_{variant}_{platform.machine()}"
    obj.mkdir(parents=True, exist_ok=True)
    base = ["g++", "-std=c++20", "-O2", "-fPIC", "-DNDEBUG", "-w", "-x", "c++", "-I", str(SHIM), "-I", str(src),
            "-include", "cuda_shim_pre.h"]
    jobs = []
    for u in UNITS:
        o = obj / (u.replace("/", "_") + ".o")
        extra = [] if u in HOST_SIDE else ["-D__CUDA_ARCH__=900"]
        jobs.append((base + extra + ["-c", str(src / u), "-o", str(o)], o))
    drv = obj / "ref_driver.o"
    if drv.exists() and drv.stat().st_mtime < DRIVER.stat().st_mtime:
        drv.unlink()
    jobs.append((base + ["-D__CUDA_ARCH__=900", "-c", str(DRIVER), "-o", str(drv)], drv))
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_compile, jobs))
    r = subprocess.run(["g++", "-shared", "-o", str(lib), *[str(j[1]) for j in jobs]], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return lib


def build() -> dict:
    OUT.mkdir(exist_ok=True)
    return {v: build_variant(v) for v in VARIANTS}


if __name__ == "__main__":
    print(build())
    sys.exit(0)
