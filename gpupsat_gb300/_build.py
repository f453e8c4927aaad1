"""Builds libgpsat.so (sm_103a kernels + C++ host code) in-tree.

nvcc compiles every .cu for sm_103a only; g++ compiles the host .cpp files;
translation units build in parallel.  Objects go to gpupsat_gb300/_build/, the
library to gpupsat_gb300/libgpsat.so.  A unit is rebuilt when it, or any
header under csrc/ or include/, is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build" / platform.machine()  # objects never cross architectures
LIB = PKG / "libgpsat.so"
CLI = PKG / "gpsat"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")))


def _stale(src: Path, obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(h.stat().st_mtime > t for h in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(parents=True, exist_ok=True)
    hdrs = _headers()
    inc = ["-I", str(CSRC), "-I", str(ROOT / "include")]
    cmds = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if _stale(src, obj, hdrs):
            cmds.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas",
                         "-v" if verbose else "-O3", *inc, "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        if src.name.startswith("cli_"):
            continue
        obj = BUILD / (src.stem + ".cpp.o")
        objs.append(obj)
        if _stale(src, obj, hdrs):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", *inc, "-I", str(cuda / "include"),
                         "-c", str(src), "-o", str(obj)])
    if cmds:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, cmds))
    stamp = BUILD / "libgpsat.stamp"
    if cmds or not LIB.exists() or not stamp.exists() or stamp.stat().st_mtime < LIB.stat().st_mtime - 1:
        _run(["g++", "-shared", "-o", str(LIB), *map(str, objs), "-L", str(cuda / "lib64"),
              "-Wl,-rpath," + str(cuda / "lib64"), "-lcudart", "-pthread"])
        stamp.write_text(platform.machine() + "\n")
    cli_src = CSRC / "cli_main.cpp"
    if cli_src.exists() and (_stale(cli_src, CLI, hdrs + [LIB]) or cmds):
        _run(["g++", "-O2", "-std=c++17", "-pthread", *inc, str(cli_src), "-o", str(CLI), "-L", str(PKG),
              "-Wl,-rpath,$ORIGIN", "-lgpsat"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
