"""ORACLE -- test infrastructure only.

CPU checkers for the gpsat GPU path.  Only tests/, __graft_entry__.smoke()
and the CPU-baseline leg of bench.py import this package; the shipped
library never does.

  bcp_ref.c   C restatement of the reference's two-watched-literal BCP in its
              own processing order (see the file header for the cited lines)
  gen.c       the benchmark workloads' seeded generators (random k-SAT,
              partial trails), restated so that the CPU side of the benchmark
              never loads the shipped library; pinned to it by a CPU test
  ref/        recipe that compiles the reference's own solver sources for the
              host (output: oracle/_ref/), used to pin the restatement
"""
from __future__ import annotations

import ctypes
import platform
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / f"liboracle_{platform.machine()}.so"
SOURCES = [HERE / "bcp_ref.c", HERE / "gen.c"]

_lib = None
_vp = ctypes.c_void_p


def build() -> Path:
    """Compiles the C restatement (gcc, portable flags, no arch tuning)."""
    if not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in SOURCES):
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-pthread", *map(str, SOURCES), "-o", str(LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        L.orc_bcp_create.restype = _vp
        L.orc_bcp_create.argtypes = [_vp, _vp, ctypes.c_int32, ctypes.c_int64]
        L.orc_bcp_destroy.argtypes = [_vp]
        L.orc_bcp_initial_watches.argtypes = [_vp, _vp, _vp]
        L.orc_bcp_run.argtypes = [_vp, _vp, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64] + [_vp] * 7
        L.orc_scan_run.argtypes = [_vp, _vp, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64] + [_vp] * 7
        L.orc_gen_random_ksat.argtypes = [ctypes.c_uint64, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, _vp]
        L.orc_gen_trails.argtypes = [ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                     ctypes.c_double, _vp, _vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def gen_random_ksat(seed: int, n_vars: int, n_clauses: int, k: int = 3):
    """Uniform random k-SAT, the same instances as the library's generator. Returns (lits, offsets)."""
    lits = np.empty(n_clauses * k, np.int32)
    if lib().orc_gen_random_ksat(seed, n_vars, n_clauses, k, _p(lits)) != 0:
        raise ValueError("gen_random_ksat: need 0 < k <= min(n_vars, 64)")
    return lits, np.arange(0, n_clauses * k + 1, k, dtype=np.int64)


def gen_trails(seed: int, n_vars: int, n_trails: int, fmin: float = 0.01, fmax: float = 0.05):
    """Random partial trails, the same as the library's generator. Returns (lits, offsets)."""
    off = np.empty(n_trails + 1, np.int64)
    if lib().orc_gen_trails(seed, n_vars, n_trails, fmin, fmax, _p(off), None) != 0:
        raise ValueError("gen_trails: need n_vars > 0, 0 <= fmin <= fmax <= 1")
    lits = np.empty(int(off[-1]), np.int32)
    if lib().orc_gen_trails(seed, n_vars, n_trails, fmin, fmax, _p(off), _p(lits)) != 0:
        raise MemoryError("gen_trails")
    return lits, off


class BCPOracle:
    """Reference-order BCP on the CPU. Clauses must be clean (length >= 2, distinct variables)."""

    def __init__(self, lits: np.ndarray, offsets: np.ndarray, n_vars: int):
        self._lits = np.ascontiguousarray(lits, dtype=np.int32)
        self._off = np.ascontiguousarray(offsets, dtype=np.int64)
        self.n_clauses = len(self._off) - 1
        self._h = lib().orc_bcp_create(_p(self._lits), _p(self._off), n_vars, self.n_clauses)
        if not self._h:
            raise ValueError("oracle rejected the formula (needs clean clauses of length >= 2)")

    def initial_watches(self):
        w1 = np.empty(self.n_clauses, np.int32)
        w2 = np.empty(self.n_clauses, np.int32)
        lib().orc_bcp_initial_watches(self._h, _p(w1), _p(w2))
        return w1, w2

    def run(self, trail_lits: np.ndarray, trail_offsets: np.ndarray, impl_cap: int = 4096, threads: int = 1,
            strategy: str = "watched") -> dict:
        """strategy "watched": the reference's two-watched-literal BCP;
        "full_scan": its full-scan clause evaluation (BASIC_SEARCH)."""
        trail_lits = np.ascontiguousarray(trail_lits, dtype=np.int32)
        trail_offsets = np.ascontiguousarray(trail_offsets, dtype=np.int64)
        T = len(trail_offsets) - 1
        out = dict(status=np.empty(T, np.int32), conflict=np.empty(T, np.int32), stop=np.empty(T, np.int32),
                   n_impl=np.empty(T, np.int64), impl_lit=np.zeros((T, impl_cap), np.int32),
                   impl_reason=np.zeros((T, impl_cap), np.int32), counters=np.zeros((T, 6), np.int64))
        fn = lib().orc_scan_run if strategy == "full_scan" else lib().orc_bcp_run
        rc = fn(self._h, _p(trail_lits), _p(trail_offsets), T, threads, impl_cap,
                               _p(out["status"]), _p(out["conflict"]), _p(out["stop"]), _p(out["n_impl"]),
                               _p(out["impl_lit"]), _p(out["impl_reason"]), _p(out["counters"]))
        if rc != 0:
            raise RuntimeError(f"oracle run failed: {rc}")
        return out

    def close(self):
        if self._h:
            lib().orc_bcp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
