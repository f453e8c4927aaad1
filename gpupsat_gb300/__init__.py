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
BCP_WATCHED, BCP_FULL_SCAN = 0, 1
BCP_NCOUNTERS = 6
BCP_COUNTER_NAMES = ("props", "watches", "clause_lits", "lookups", "implications", "trail_lits")

_lib = None

_c_i32p = ctypes.POINTER(ctypes.c_int32)
_c_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p


DECIDE_VSIDS, DECIDE_LAST_FREE = 0, 1
RESTART_NONE, RESTART_LUBY, RESTART_GEOMETRIC = 0, 1, 2
SOLVE_STAT_NAMES = ("conflicts", "decisions", "propagations", "restarts", "learnts", "reductions", "rebuilds",
                    "flags", "jobs")


class SolveOptions(ctypes.Structure):
    _fields_ = [("decide", ctypes.c_int32), ("restart", ctypes.c_int32), ("restart_base", ctypes.c_int32),
                ("restart_factor", ctypes.c_float), ("var_decay", ctypes.c_float),
                ("learnt_first", ctypes.c_int32), ("learnt_inc", ctypes.c_int32), ("minimize", ctypes.c_int32),
                ("conflict_budget", ctypes.c_int64), ("phase_init", ctypes.c_int32),
                ("max_slots", ctypes.c_int32), ("log_participation", ctypes.c_int32),
                ("proof_words", ctypes.c_int32), ("reserved", ctypes.c_int32 * 4)]


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
        "gpsat_bcp_set_active_slots": (ctypes.c_int, [_vp, ctypes.c_int32]),
        "gpsat_bcp_set_strategy": (ctypes.c_int, [_vp, ctypes.c_int32]),
        "gpsat_bcp_set_window": (ctypes.c_int, [_vp, ctypes.c_int32]),
        "gpsat_bcp_set_order_pivot": (ctypes.c_int, [_vp, ctypes.c_int64]),
        "gpsat_bcp_window_slots": (ctypes.c_int, [_vp, ctypes.c_int32, _c_i32p]),
        "gpsat_bcp_run_device": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int32] + [_vp] * 8),
        "gpsat_bcp_run_host": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int32] + [_vp] * 7),
        "gpsat_bcp_run_static": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64, _vp, _vp, ctypes.c_int32]
                                 + [_vp] * 8),
        "gpsat_solve_options_default": (ctypes.c_int, [ctypes.POINTER(SolveOptions)]),
        "gpsat_batch_create": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int32, ctypes.POINTER(_vp)]),
        "gpsat_batch_destroy": (ctypes.c_int, [_vp]),
        "gpsat_batch_info": (ctypes.c_int, [_vp, _c_i32p, _c_i64p, _c_i32p, _c_i64p]),
        "gpsat_batch_set_seeds": (ctypes.c_int, [_vp, _vp, _vp]),
        "gpsat_batch_solve": (ctypes.c_int, [_vp, ctypes.POINTER(SolveOptions), _vp, _vp, _vp, ctypes.c_int32]
                              + [_vp] * 5),
        "gpsat_check_model": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, ctypes.c_int32, _c_i64p]),
        "gpsat_batch_proof": (ctypes.c_int, [_vp, ctypes.c_int32, _c_i32p, _vp, ctypes.c_int64, _c_i64p]),
        "gpsat_check_rup": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp, ctypes.c_int32, _vp,
                                           ctypes.c_int64, _c_i64p]),
        "gpsat_gen_random_ksat": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, _vp]),
        "gpsat_gen_trails": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                            ctypes.c_double, _vp, _vp]),
        "gpsat_dimacs_parse": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int64, _c_i32p, _c_i64p, _c_i64p, _c_i32p,
                                              _c_i64p, _vp, _vp]),
        "gpsat_gen_planted": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.c_double, _vp, _vp]),
        # learned seeding kernels (device pointers)
        "gpsat_gnn_mm": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, _vp, ctypes.c_int32,
                                        ctypes.c_int32, _vp, ctypes.c_int32, _vp, ctypes.c_int32, _vp, _vp]),
        "gpsat_gnn_wgrad": (ctypes.c_int, [_vp, ctypes.c_int32, _vp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                           _vp, _vp, _vp]),
        "gpsat_gnn_gather": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp, ctypes.c_int32, _vp, _vp,
                                            ctypes.c_int32, _vp, ctypes.c_int32, ctypes.c_int32, _vp]),
        "gpsat_gnn_gather_split": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, ctypes.c_int32, _vp, _vp, _vp,
                                                  ctypes.c_int32, _vp]),
        "gpsat_gnn_relu_bwd": (ctypes.c_int, [_vp, ctypes.c_int32, _vp, ctypes.c_int32, ctypes.c_int64, _vp,
                                              ctypes.c_int32, _vp]),
        "gpsat_gnn_colsum": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int64, _vp, _vp]),
        "gpsat_gnn_broadcast": (ctypes.c_int, [_vp, ctypes.c_int64, _vp, ctypes.c_int32, _vp]),
        "gpsat_gnn_head": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int64] + [_vp] * 8 + [ctypes.c_int32, _vp, _vp,
                                                                                               _vp]),
        "gpsat_gnn_adam": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int64, ctypes.c_float, ctypes.c_float,
                                          ctypes.c_float, ctypes.c_float, ctypes.c_int64, _vp]),
        "gpsat_gnn_pack": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp, ctypes.c_int32, _vp]),
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


def parse_dimacs(text: str | bytes) -> dict:
    """DIMACS CNF text -> dict(lits, offsets, n_vars, header_vars, header_clauses)
    (gpsat_dimacs_parse; n_vars is the highest variable found, as the
    reference's reader sets it)."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    nv, nc, nl, hv, hc = (ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int64())
    L = lib()
    check(L.gpsat_dimacs_parse(data, len(data), ctypes.byref(nv), ctypes.byref(nc), ctypes.byref(nl),
                               ctypes.byref(hv), ctypes.byref(hc), None, None))
    lits = np.empty(nl.value, np.int32)
    off = np.empty(nc.value + 1, np.int64)
    check(L.gpsat_dimacs_parse(data, len(data), ctypes.byref(nv), ctypes.byref(nc), ctypes.byref(nl),
                               ctypes.byref(hv), ctypes.byref(hc), _p(lits), _p(off)))
    return dict(lits=lits, offsets=off, n_vars=nv.value, header_vars=hv.value, header_clauses=hc.value)


def gen_planted(seed: int, n_vars: int, n_clauses: int, k: int = 3, communities: int = 40, p_in: float = 0.9):
    """Planted k-SAT with community structure. Returns (lits, offsets, planted)
    where planted[v-1] = +1/-1 is the hidden satisfying assignment."""
    lits = np.empty(n_clauses * k, dtype=np.int32)
    planted = np.empty(n_vars, dtype=np.int8)
    check(lib().gpsat_gen_planted(seed, n_vars, n_clauses, k, communities, p_in, _p(lits), _p(planted)))
    return lits, np.arange(0, n_clauses * k + 1, k, dtype=np.int64), planted


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
    """Reference-order two-watched-literal BCP over many partial trails (one thread block per trail)."""

    def __init__(self, formula: Formula, max_slots: int = 0, impl_cap: int = 4096, arena_cap: int = 0):
        self.formula = formula
        self.impl_cap = impl_cap
        self._h = _vp()
        check(lib().gpsat_bcp_create(formula.handle, max_slots, impl_cap, arena_cap, ctypes.byref(self._h)))
        self.active = 0
        self.pivot = 0
        self.window = 128
        self.strategy = "watched"

    def info(self) -> dict:
        s, b = ctypes.c_int32(), ctypes.c_int64()
        check(lib().gpsat_bcp_info(self._h, ctypes.byref(s), ctypes.byref(b)))
        return dict(slots=s.value, device_bytes=b.value)

    def window_slots(self, entries: int) -> int:
        """Trails the window width keeps in flight at most."""
        n = ctypes.c_int32()
        check(lib().gpsat_bcp_window_slots(self._h, int(entries), ctypes.byref(n)))
        return n.value

    def set_window(self, entries: int) -> None:
        """Watch entries per round of the two-watched-literal kernel (64, 128
        or 256); outputs do not depend on it."""
        check(lib().gpsat_bcp_set_window(self._h, int(entries)))
        self.window = int(entries)

    def tune(self, trail_lits, trail_offsets, out: dict, stream: int, windows=(128, 256, 64),
             fractions=(1.0, 0.75, 0.5), pivots=(0.0, 0.1, 0.2, 0.3, 0.4)):
        """The BCP autotuner: times one run_device launch of these trails (after
        one untimed launch) for every window width and, at each width, every
        fraction of the slots that width keeps resident, then, at the fastest
        pair, the processing order's pivot at each quantile of the trail
        lengths in `pivots` (0: shortest first); keeps the fastest setting.
        Returns {(window, active slots, pivot): ms}.  Outputs do not depend on
        the setting; `out` holds the last launch's results."""
        import torch
        st = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
        slots = self.info()["slots"]
        times = {}

        def timed(key):
            self.run_device(trail_lits, trail_offsets, out, stream=stream)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            self.run_device(trail_lits, trail_offsets, out, stream=stream)
            b.record(st)
            b.synchronize()
            times[key] = a.elapsed_time(b)

        self.set_order_pivot(0)
        for w in windows:
            self.set_window(w)
            per = self.window_slots(w)
            for f in fractions:
                n = max(4, int(per * f) // 4 * 4)
                if n > slots:
                    continue
                self.set_active_slots(n)
                timed((w, n, 0))
        (w, n, _) = min(times, key=times.get)
        self.set_window(w)
        self.set_active_slots(n)
        offs = trail_offsets.cpu().numpy() if hasattr(trail_offsets, "cpu") else np.asarray(trail_offsets)
        lens = np.diff(offs.astype(np.int64))
        for q in pivots:
            p = int(np.quantile(lens, q)) if q > 0 and len(lens) else 0
            if p == 0 or (w, n, p) in times:
                continue
            self.set_order_pivot(p)
            timed((w, n, p))
        (w, n, p) = min(times, key=times.get)
        self.set_window(w)
        self.set_active_slots(n)
        self.set_order_pivot(p)
        return times

    def set_order_pivot(self, pivot: int) -> None:
        """Later runs start the trails whose literal count is nearest `pivot`
        first (0: shortest first); outputs do not depend on it."""
        check(lib().gpsat_bcp_set_order_pivot(self._h, int(pivot)))
        self.pivot = int(pivot)

    def set_strategy(self, strategy: str) -> None:
        """"watched" (two watched literals, the default) or "full_scan" (the
        reference's full-scan clause evaluation) for the runs that follow."""
        code = {"watched": BCP_WATCHED, "full_scan": BCP_FULL_SCAN}.get(strategy, -1)
        check(lib().gpsat_bcp_set_strategy(self._h, code))
        self.strategy = strategy

    def set_active_slots(self, n: int) -> None:
        """Later runs use at most n slots (0 = all); outputs do not depend on it."""
        check(lib().gpsat_bcp_set_active_slots(self._h, int(n)))
        self.active = int(n)

    def host_outputs(self, n_trails: int, counters: bool = True, alloc=np.zeros) -> dict:
        """Output arrays for run_host (alloc may return pinned memory, e.g. numpy
        views of torch.empty(..., pin_memory=True))."""
        T = n_trails
        return dict(status=alloc(T, np.int32), conflict=alloc(T, np.int32), stop=alloc(T, np.int32),
                    n_impl=alloc(T, np.int64), impl_lit=alloc((T, self.impl_cap), np.int32),
                    impl_reason=alloc((T, self.impl_cap), np.int32),
                    counters=alloc((T, BCP_NCOUNTERS), np.int64) if counters else None)

    def run_host(self, trail_lits: np.ndarray, trail_offsets: np.ndarray, counters: bool = True,
                 out: dict | None = None) -> dict:
        """Host buffers in and out (gpsat_bcp_run_host).  `out` (from host_outputs)
        is reused when given; entries of impl_lit / impl_reason past n_impl[t]
        are left as they were."""
        trail_lits = np.ascontiguousarray(trail_lits, dtype=np.int32)
        trail_offsets = np.ascontiguousarray(trail_offsets, dtype=np.int64)
        T = len(trail_offsets) - 1
        if T < 0 or (T > 0 and trail_offsets[-1] > len(trail_lits)):
            raise ValueError("run_host: trail_offsets must have n_trails + 1 entries ending within trail_lits")
        if out is None:
            out = self.host_outputs(T, counters)
        else:
            for k, dt in (("status", np.int32), ("conflict", np.int32), ("stop", np.int32), ("n_impl", np.int64),
                          ("impl_lit", np.int32), ("impl_reason", np.int32)):
                a = out[k]
                if a.dtype != dt or a.shape[0] != T or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"run_host: out[{k!r}] must be a contiguous {np.dtype(dt)} array of {T} rows")
            if out["impl_lit"].shape[1] != self.impl_cap or out["impl_reason"].shape[1] != self.impl_cap:
                raise ValueError("run_host: implication arrays must have impl_cap columns")
        check(lib().gpsat_bcp_run_host(self._h, _p(trail_lits), _p(trail_offsets), T, _p(out["status"]),
                                       _p(out["conflict"]), _p(out["stop"]), _p(out["n_impl"]),
                                       _p(out["impl_lit"]), _p(out["impl_reason"]), _p(out["counters"])))
        return out

    def run_device(self, trail_lits, trail_offsets, out: dict, stream: int | None = None) -> None:
        """Device buffers (torch tensors); `out` holds status, conflict, stop, n_impl, impl_lit, impl_reason, counters."""
        T = trail_offsets.numel() - 1
        _check_device_outputs(out, T, self.impl_cap, trail_lits, trail_offsets)
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


def _check_device_outputs(out: dict, T: int, impl_cap: int, trail_lits, trail_offsets) -> None:
    """The kernel writes trail t's implications at t * impl_cap: every output
    must be a contiguous device tensor of the right dtype and shape, on the
    trails' device, or the call is refused before it reaches the library."""
    import torch
    dev = trail_offsets.device
    if trail_offsets.dtype != torch.int64 or trail_lits.dtype != torch.int32 or trail_lits.device != dev:
        raise GpsatError(-1, "trail_lits must be int32 and trail_offsets int64, on one device")
    want = {"status": (torch.int32, (T,)), "conflict": (torch.int32, (T,)), "stop": (torch.int32, (T,)),
            "n_impl": (torch.int64, (T,)), "impl_lit": (torch.int32, (T, impl_cap)),
            "impl_reason": (torch.int32, (T, impl_cap))}
    if out.get("counters") is not None:
        want["counters"] = (torch.int64, (T, BCP_NCOUNTERS))
    for k, (dt, shape) in want.items():
        a = out.get(k)
        if a is None or a.dtype != dt or tuple(a.shape) != shape or not a.is_contiguous() or a.device != dev:
            raise GpsatError(-1, f"out[{k!r}] must be a contiguous {dt} tensor of shape {shape} on {dev}")


def bcp_run_static(formula: Formula, trail_lits, trail_offsets, out: dict, impl_cap: int, arena_cap: int = 0,
                   stream: int | None = None) -> None:
    """gpsat_bcp_run_static: BCP with the library's fixed device scratch (no
    allocation inside the call).  Device buffers (torch tensors) as in
    BCPBatch.run_device; the formula must already be on the device (creating
    a BCPBatch on it uploads it)."""
    T = trail_offsets.numel() - 1
    _check_device_outputs(out, T, impl_cap, trail_lits, trail_offsets)
    check(lib().gpsat_bcp_run_static(formula.handle, impl_cap, arena_cap, _p(trail_lits), _p(trail_offsets), T,
                                     _p(out["status"]), _p(out["conflict"]), _p(out["stop"]), _p(out["n_impl"]),
                                     _p(out["impl_lit"]), _p(out["impl_reason"]), _p(out.get("counters")), stream))


# ---------------------------------------------------------------- CDCL solving
def solve_options(**kw) -> SolveOptions:
    o = SolveOptions()
    check(lib().gpsat_solve_options_default(ctypes.byref(o)))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def check_model(lits: np.ndarray, offsets: np.ndarray, model: np.ndarray, n_vars: int) -> bool:
    """Host model check (independent of the device checker)."""
    lits = np.ascontiguousarray(lits, np.int32)
    offsets = np.ascontiguousarray(offsets, np.int64)
    model = np.ascontiguousarray(model, np.int8)
    bad = ctypes.c_int64(-1)
    rc = lib().gpsat_check_model(_p(lits), _p(offsets), len(offsets) - 1, _p(model), n_vars, ctypes.byref(bad))
    if rc < 0:
        check(rc)
    return rc == 1


def check_rup(lits: np.ndarray, offsets: np.ndarray, n_vars: int, proof: np.ndarray, assumptions=None) -> tuple:
    """Host RUP check of an UNSAT proof log (gpsat_check_rup): (refuted, failed_step)."""
    lits = np.ascontiguousarray(lits, np.int32)
    offsets = np.ascontiguousarray(offsets, np.int64)
    proof = np.ascontiguousarray(proof, np.int32)
    a = None if assumptions is None or len(assumptions) == 0 else np.ascontiguousarray(assumptions, np.int32)
    step = ctypes.c_int64(-1)
    rc = lib().gpsat_check_rup(_p(lits), _p(offsets), len(offsets) - 1, n_vars, _p(a), 0 if a is None else len(a),
                               _p(proof) if len(proof) else None, len(proof), ctypes.byref(step))
    if rc < 0:
        check(rc)
    return rc == 1, step.value


class Batch:
    """Many formulas solved on the GPU by the device CDCL solver (one warp per job)."""

    def __init__(self, formulas, n_vars):
        """formulas: list of (lits, offsets) CSR pairs (DIMACS literals); n_vars: list of ints."""
        self.n_vars = np.asarray(n_vars, np.int32)
        offs = [np.asarray(o, np.int64) for _, o in formulas]
        lits = np.concatenate([np.asarray(l, np.int32) for l, _ in formulas]) if formulas else np.zeros(0, np.int32)
        coff = np.zeros(sum(len(o) - 1 for o in offs) + 1, np.int64)
        foff = np.zeros(len(formulas) + 1, np.int64)
        c = 0
        base = 0
        for i, o in enumerate(offs):
            k = len(o) - 1
            coff[c + 1:c + k + 1] = o[1:] + base
            base += int(o[-1])
            c += k
            foff[i + 1] = c
        self.clause_lits, self.clause_offsets, self.formula_offsets = lits, coff, foff
        self.var_off = np.zeros(len(formulas) + 1, np.int64)
        self.var_off[1:] = np.cumsum(self.n_vars)
        self._h = _vp()
        check(lib().gpsat_batch_create(_p(lits), _p(coff), _p(foff), _p(self.n_vars), len(formulas),
                                       ctypes.byref(self._h)))

    @property
    def n_formulas(self) -> int:
        return len(self.n_vars)

    def formula(self, f: int):
        c0, c1 = self.formula_offsets[f], self.formula_offsets[f + 1]
        o = self.clause_offsets[c0:c1 + 1]
        return self.clause_lits[o[0]:o[-1]], o - o[0]

    def info(self) -> dict:
        nf, tv, s, wb = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int64()
        check(lib().gpsat_batch_info(self._h, ctypes.byref(nf), ctypes.byref(tv), ctypes.byref(s), ctypes.byref(wb)))
        return dict(n_formulas=nf.value, total_vars=tv.value, slots=s.value, workspace_bytes=wb.value)

    def set_seeds(self, activity=None, phase=None) -> None:
        a = None if activity is None else np.ascontiguousarray(activity, np.float32)
        p = None if phase is None else np.ascontiguousarray(phase, np.int8)
        check(lib().gpsat_batch_set_seeds(self._h, _p(a), _p(p)))

    def solve(self, options: SolveOptions | None = None, jobs=None, participation: bool | int = False,
              proof_words: int = 0) -> dict:
        """jobs: None, or (job_formula int32[J], cube_offsets int64[J+1], cube_lits int32[...]).
        participation: True / 1 logs per-variable conflict participation
        (out["participation"]); 2 also learnt-clause occurrences
        (out["learnt_occurrences"])."""
        F = self.n_formulas
        V = int(self.var_off[-1])
        o = SolveOptions.from_buffer_copy(options) if options is not None else solve_options()
        level = int(participation)
        if level:
            o.log_participation = level
        if proof_words:
            o.proof_words = int(proof_words)
        out = dict(verdict=np.zeros(F, np.int32), model=np.zeros(V, np.int8),
                   stats=np.zeros((F, 9), np.int64), model_ok=np.zeros(F, np.int32),
                   participation=np.zeros(V * (2 if level >= 2 else 1), np.int32) if level else None)
        jf = co = cl = None
        nj = 0
        if jobs is not None:
            jf = np.ascontiguousarray(jobs[0], np.int32)
            co = np.ascontiguousarray(jobs[1], np.int64)
            cl = np.ascontiguousarray(jobs[2], np.int32)
            nj = len(jf)
            if len(co) != nj + 1 or (nj and (co[0] < 0 or (np.diff(co) < 0).any() or co[-1] > len(cl))):
                raise GpsatError(-1, "cube_offsets must hold len(job_formula) + 1 non-decreasing offsets into cube_lits")
        check(lib().gpsat_batch_solve(self._h, ctypes.byref(o), _p(jf), _p(co), _p(cl), nj, _p(out["verdict"]),
                                      _p(out["model"]), _p(out["stats"]), _p(out["model_ok"]),
                                      _p(out["participation"])))
        if level >= 2:
            out["learnt_occurrences"] = out["participation"][V:]
            out["participation"] = out["participation"][:V]
        return out

    def proof(self, job: int) -> tuple:
        """(job verdict, proof log as int32 words, or None when it overflowed)
        of a job of the last solve made with proof_words > 0 (gpsat_batch_proof)."""
        v, n = ctypes.c_int32(), ctypes.c_int64()
        check(lib().gpsat_batch_proof(self._h, job, ctypes.byref(v), None, 0, ctypes.byref(n)))
        if n.value < 0:
            return v.value, None
        w = np.empty(max(n.value, 1), np.int32)
        check(lib().gpsat_batch_proof(self._h, job, ctypes.byref(v), _p(w), n.value, ctypes.byref(n)))
        return v.value, w[:n.value]

    def certify_unsat(self, verdicts, jobs=None, threads: int | None = None) -> dict:
        """Checks the proof log of every UNSAT job of the last solve (made with
        proof_words > 0) against the original clauses and the job's cube, on
        the host, several jobs at a time.  Returns {caller job: (ok, failed
        step or reason)} for the jobs whose own verdict is UNSAT."""
        import concurrent.futures as cf
        if jobs is None:
            todo = [(int(f), int(f), None) for f in np.nonzero(np.asarray(verdicts) == UNSAT)[0]]
        else:
            jf, co, cl = jobs
            todo = [(j, int(jf[j]), cl[co[j]:co[j + 1]]) for j in range(len(jf))]

        def one(item):
            j, f, cube = item
            v, words = self.proof(j)
            if v != UNSAT:
                return j, None
            if words is None:
                return j, (False, "log overflowed")
            lits, off = self.formula(f)
            return j, check_rup(lits, off, int(self.n_vars[f]), words, cube)

        out = {}
        with cf.ThreadPoolExecutor(threads or os.cpu_count() or 4) as ex:
            for j, r in ex.map(one, todo):
                if r is not None:
                    out[j] = r
        return out

    def model_of(self, out: dict, f: int) -> np.ndarray:
        return out["model"][self.var_off[f]:self.var_off[f + 1]]

    def close(self) -> None:
        if self._h:
            lib().gpsat_batch_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
