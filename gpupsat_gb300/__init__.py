"""gpsat: GB300-native CDCL SAT engine -- Python bindings over the C ABI.

The compute path is libgpsat.so (hand-written sm_103a kernels + C++ host
code, declared in include/gpsat.h).  This module only loads it with ctypes
and moves numpy / torch buffers across; there is no Python fallback: if the
library is missing, importing a handle raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libgpsat.so"

OK = 0
UNKNOWN, SAT, UNSAT = 0, 10, 20
BCP_NO_CONFLICT, BCP_CONFLICT, BCP_OVERFLOW, BCP_BAD_TRAIL = 0, 1, -1, -2
BCP_NCOUNTERS = 6
BCP_COUNTER_NAMES = ("props", "watches", "clause_lits", "lookups", "implications", "trail_lits")

_lib = None

_c_i32p = ctypes.POINTER(ctypes.c_int32)
_c_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p


class GpsatError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gpsat error {code}: {msg}")
        self.code = code


def lib() -> ctypes.CDLL:
    """Loads libgpsat.so (built by gpupsat_gb300._build); raises if absent."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise GpsatError(-100, f"{LIB_PATH} is not built; run __graft_entry__.build()")
        L = ctypes.CDLL(str(LIB_PATH))
        _declare(L)
        _lib = L
    return _lib


def _declare(L: ctypes.CDLL) -> None:
    sig = {
        "gpsat_version": (ctypes.c_char_p, []),
        "gpsat_error_string": (ctypes.c_char_p, [ctypes.c_int]),
        "gpsat_last_error": (ctypes.c_char_p, []),
        "gpsat_device_count": (ctypes.c_int, [_c_i32p]),
        "gpsat_formula_create": (ctypes.c_int, [_vp, _vp, ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(_vp)]),
        "gpsat_formula_destroy": (ctypes.c_int, [_vp]),
        "gpsat_formula_info": (ctypes.c_int, [_vp, _c_i32p, _c_i64p, _c_i64p, _c_i32p, _c_i64p]),
        "gpsat_formula_export": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
        "gpsat_bcp_create": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(_vp)]),
        "gpsat_bcp_destroy": (ctypes.c_int, [_vp]),
        "gpsat_bcp_info": (ctypes.c_int, [_vp, _c_i32p, _c_i64p]),
        "gpsat_bcp_run_device": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int32] + [_vp] * 8),
        "gpsat_bcp_run_host": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int32] + [_vp] * 7),
        "gpsat_gen_random_ksat": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, _vp]),
        "gpsat_gen_trails": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                            ctypes.c_double, _vp, _vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def check(rc: int) -> None:
    if rc != OK:
        L = lib()
        raise GpsatError(rc, f"{L.gpsat_error_string(rc).decode()}: {L.gpsat_last_error().decode()}")


def _p(a) -> int | None:
    """Address of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    return a.data_ptr()


def version() -> str:
    return lib().gpsat_version().decode()


def device_count() -> int:
    n = ctypes.c_int32(0)
    check(lib().gpsat_device_count(ctypes.byref(n)))
    return n.value


# ---------------------------------------------------------------- generators
def gen_random_ksat(seed: int, n_vars: int, n_clauses: int, k: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """Uniform random k-SAT (distinct variables, fair signs). Returns (lits, offsets)."""
    lits = np.empty(n_clauses * k, dtype=np.int32)
    check(lib().gpsat_gen_random_ksat(seed, n_vars, n_clauses, k, _p(lits)))
    return lits, np.arange(0, n_clauses * k + 1, k, dtype=np.int64)


def gen_trails(seed: int, n_vars: int, n_trails: int, fmin: float = 0.01, fmax: float = 0.05):
    """Random partial trails of distinct variables. Returns (lits, offsets)."""
    off = np.empty(n_trails + 1, dtype=np.int64)
    check(lib().gpsat_gen_trails(seed, n_vars, n_trails, fmin, fmax, _p(off), None))
    lits = np.empty(int(off[-1]), dtype=np.int32)
    check(lib().gpsat_gen_trails(seed, n_vars, n_trails, fmin, fmax, _p(off), _p(lits)))
    return lits, off


def clauses_to_csr(clauses) -> tuple[np.ndarray, np.ndarray]:
    off = np.zeros(len(clauses) + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(c) for c in clauses])
    lits = np.fromiter((x for c in clauses for x in c), dtype=np.int32, count=int(off[-1]))
    return lits, off


# ---------------------------------------------------------------- formula
class Formula:
    """A preprocessed formula (reference preprocessing + initial watches); device copy made on first use."""

    def __init__(self, lits: np.ndarray, offsets: np.ndarray, n_vars: int):
        self._h = _vp()
        lits = np.ascontiguousarray(lits, dtype=np.int32)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        check(lib().gpsat_formula_create(_p(lits), _p(offsets), n_vars, len(offsets) - 1, ctypes.byref(self._h)))

    @classmethod
    def from_clauses(cls, clauses, n_vars: int | None = None) -> "Formula":
        lits, off = clauses_to_csr(clauses)
        if n_vars is None:
            n_vars = int(np.abs(lits).max()) if len(lits) else 1
        return cls(lits, off, n_vars)

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        nv, nc, nl, vd, ns = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int64()
        check(lib().gpsat_formula_info(self._h, ctypes.byref(nv), ctypes.byref(nc), ctypes.byref(nl),
                                       ctypes.byref(vd), ctypes.byref(ns)))
        return dict(n_vars=nv.value, n_clauses=nc.value, n_lits=nl.value, verdict=vd.value, n_solved=ns.value)

    def export(self) -> dict:
        i = self.info()
        lits = np.empty(i["n_lits"], np.int32)
        off = np.empty(i["n_clauses"] + 1, np.int64)
        solved = np.empty(i["n_solved"], np.int32)
        w1 = np.empty(i["n_clauses"], np.int32)
        w2 = np.empty(i["n_clauses"], np.int32)
        check(lib().gpsat_formula_export(self._h, _p(lits), _p(off), _p(solved), _p(w1), _p(w2)))
        return dict(lits=lits, offsets=off, solved=solved, watch1=w1, watch2=w2, **i)

    def close(self) -> None:
        if self._h:
            lib().gpsat_formula_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- BCP batch
class BCPBatch:
    """Reference-order two-watched-literal BCP over many partial trails (one warp per trail)."""

    def __init__(self, formula: Formula, max_slots: int = 0, impl_cap: int = 4096, arena_cap: int = 0):
        self.formula = formula
        self.impl_cap = impl_cap
        self._h = _vp()
        check(lib().gpsat_bcp_create(formula.handle, max_slots, impl_cap, arena_cap, ctypes.byref(self._h)))

    def info(self) -> dict:
        s, b = ctypes.c_int32(), ctypes.c_int64()
        check(lib().gpsat_bcp_info(self._h, ctypes.byref(s), ctypes.byref(b)))
        return dict(slots=s.value, device_bytes=b.value)

    def run_host(self, trail_lits: np.ndarray, trail_offsets: np.ndarray, counters: bool = True) -> dict:
        trail_lits = np.ascontiguousarray(trail_lits, dtype=np.int32)
        trail_offsets = np.ascontiguousarray(trail_offsets, dtype=np.int64)
        T = len(trail_offsets) - 1
        out = dict(
            status=np.empty(T, np.int32), conflict=np.empty(T, np.int32), stop=np.empty(T, np.int32),
            n_impl=np.empty(T, np.int64), impl_lit=np.zeros((T, self.impl_cap), np.int32),
            impl_reason=np.zeros((T, self.impl_cap), np.int32),
            counters=np.zeros((T, BCP_NCOUNTERS), np.int64) if counters else None)
        check(lib().gpsat_bcp_run_host(self._h, _p(trail_lits), _p(trail_offsets), T, _p(out["status"]),
                                       _p(out["conflict"]), _p(out["stop"]), _p(out["n_impl"]),
                                       _p(out["impl_lit"]), _p(out["impl_reason"]), _p(out["counters"])))
        return out

    def run_device(self, trail_lits, trail_offsets, out: dict, stream: int | None = None) -> None:
        """Device buffers (torch tensors); `out` holds status, conflict, stop, n_impl, impl_lit, impl_reason, counters."""
        T = trail_offsets.numel() - 1
        check(lib().gpsat_bcp_run_device(self._h, _p(trail_lits), _p(trail_offsets), T, _p(out["status"]),
                                         _p(out["conflict"]), _p(out["stop"]), _p(out["n_impl"]),
                                         _p(out["impl_lit"]), _p(out["impl_reason"]), _p(out.get("counters")),
                                         stream))

    def close(self) -> None:
        if self._h:
            lib().gpsat_bcp_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
