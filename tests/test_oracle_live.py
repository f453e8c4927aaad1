"""CPU: the oracle against the reference itself on freshly generated cases.

The golden fixtures pin the oracle on recorded cases; these tests run the
reference's own BCP (`WatchedClausesList::new_decision` driven as
`ConflictAnalyzerWithWatchedLits::set_assumptions`, oracle/ref/ref_driver.cpp
`ref_bcp`) and its full-scan evaluation (`ConflictAnalyzer::
propagate_all_clauses`, `ref_scan`), compiled for the host from the
reference's sources (oracle/ref/build_ref.py), beside the oracle on seeded
formulas of clause widths 2 to 7, mixed widths up to 21 and long clauses of
10 to 14 literals, with ragged trails that hold the edge cases the
reference's trail application has: an empty trail, a repeated literal, a
variable given both signs.  Skipped where the host build of the reference is
not present."""
import ctypes
import platform

import numpy as np
import pytest

from conftest import compare_bcp

vp = ctypes.c_void_p


@pytest.fixture(scope="module")
def ref():
    from oracle.ref import build_ref
    lib = build_ref.OUT / f"libref_stock_{platform.machine()}.so"
    if not lib.exists():
        try:
            build_ref.build()
        except (OSError, RuntimeError) as e:
            pytest.skip(f"host build of the reference not present: {e}")
    L = ctypes.CDLL(str(lib))
    L.ref_bcp.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64, vp, ctypes.c_int64, ctypes.c_int64] + [vp] * 5
    L.ref_scan.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64, vp, ctypes.c_int64, ctypes.c_int64, vp, vp, vp]
    return L


def _p(a):
    return a.ctypes.data


def ref_run(L, lits, off, n, tl, to, cap, strategy):
    """Each trail through the reference's own entry (one formula set-up per
    trail, as the reference's solver does per assumption set)."""
    T = len(to) - 1
    out = dict(status=np.zeros(T, np.int32), conflict=np.zeros(T, np.int32), stop=np.zeros(T, np.int32),
               n_impl=np.zeros(T, np.int64), impl_lit=np.zeros((T, cap), np.int32),
               impl_reason=np.zeros((T, cap), np.int32))
    for t in range(T):
        tr = np.ascontiguousarray(tl[to[t]:to[t + 1]])
        a, b = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
        k1, c1, s1 = np.zeros(1, np.int64), np.zeros(1, np.int32), np.zeros(1, np.int32)
        if strategy == "watched":
            rc = L.ref_bcp(_p(lits), _p(off), n, len(off) - 1, _p(tr), len(tr), cap, _p(a), _p(b), _p(k1), _p(c1),
                           _p(s1))
        else:
            rc = L.ref_scan(_p(lits), _p(off), n, len(off) - 1, _p(tr), len(tr), cap, _p(a), _p(k1), _p(c1))
        assert rc != -3, "the reference's preprocessing decided a generated formula"
        out["status"][t] = rc
        out["conflict"][t], out["stop"][t], out["n_impl"][t] = c1[0], s1[0], k1[0]
        out["impl_lit"][t], out["impl_reason"][t] = a, b
    return out


def make_trails(rng, n, T, fmax):
    """Ragged trails of distinct variables, with the edge cases in the first four."""
    tls, tos = [], [0]
    for t in range(T):
        f = rng.uniform(0.01, fmax)
        vs = rng.choice(np.arange(1, n + 1), size=max(1, int(f * n)), replace=False)
        tr = np.where(rng.random(len(vs)) < 0.5, vs, -vs).astype(np.int32)
        if t == 0:
            tr = tr[:0]                                   # empty trail
        elif t == 1:
            tr = np.concatenate([tr, tr[:1]])             # a literal repeated at the end
        elif t == 2:
            tr = np.concatenate([tr, -tr[:1]])            # a variable given both signs
        elif t == 3:
            tr = np.concatenate([tr[:1], tr, tr[:2]])     # repeats at both ends
        tls.append(tr)
        tos.append(tos[-1] + len(tr))
    return np.concatenate(tls).astype(np.int32), np.array(tos, np.int64)


# (k, n, clauses per variable, largest trail fraction)
SHAPES = [(2, 40, 1.0, 0.5), (2, 300, 0.9, 0.1), (3, 60, 4.26, 0.5), (3, 600, 4.26, 0.2), (3, 1500, 3.5, 0.1),
          (4, 80, 9.9, 0.4), (5, 100, 21.0, 0.75), (7, 40, 60.0, 0.85)]


def mixed_formula(seed, n, m, widths, bias):
    """Clauses of the given widths on distinct variables; with bias > 0 a
    literal is true under a hidden assignment only with probability bias and
    the trails below follow that assignment, so long clauses also become unit
    and conflicting."""
    rng = np.random.default_rng(seed)
    hidden = rng.random(n + 1) < 0.5
    cls = []
    for _ in range(m):
        vs = rng.choice(np.arange(1, n + 1), size=int(rng.choice(widths)), replace=False)
        pos = hidden[vs] == (rng.random(len(vs)) < bias) if bias > 0 else rng.random(len(vs)) < 0.5
        cls.append(np.where(pos, vs, -vs))
    off = np.zeros(m + 1, np.int64)
    off[1:] = np.cumsum([len(c) for c in cls])
    return np.concatenate(cls).astype(np.int32), off, hidden


@pytest.mark.parametrize("strategy", ["watched", "full_scan"])
@pytest.mark.parametrize("n,m,widths,bias,fmax", [(120, 400, (2, 2, 3, 3, 3, 4, 6, 9), 0.0, 0.1),
                                                  (80, 400, tuple(range(10, 15)), 0.12, 0.9),
                                                  (300, 900, (2, 3, 5, 8, 13, 21), 0.2, 0.3)])
def test_oracle_matches_the_reference_on_mixed_widths(orc, ref, strategy, n, m, widths, bias, fmax):
    seed = n + m
    lits, off, hidden = mixed_formula(seed, n, m, widths, bias)
    rng = np.random.default_rng(seed + 1)
    tl, to = make_trails(rng, n, 12, fmax)
    if bias:
        # trails mostly follow the hidden assignment (4% of signs flipped)
        v = np.abs(tl)
        follow = hidden[v] != (rng.random(len(v)) < 0.04)
        tl = np.where(follow, v, -v).astype(np.int32)
        tl[to[2] + (to[3] - to[2]) - 1] = -tl[to[2]]        # keep trail 2's contradiction
        tl[to[1] + (to[2] - to[1]) - 1] = tl[to[1]]         # and trail 1's repeat
        tl[to[3]] = tl[to[3] + 1]                           # and trail 3's
    cap = n + 8
    r = ref_run(ref, lits, off, n, tl, to, cap, strategy)
    o = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=cap, strategy=strategy)
    assert r["status"][2] == -2 and r["n_impl"].sum() > 0 and (r["status"] == 1).any()
    assert (r["status"] == 0).sum() > 1
    for t in range(len(to) - 1):
        kk = int(r["n_impl"][t])
        assert (o["status"][t], o["conflict"][t], o["n_impl"][t]) == (r["status"][t], r["conflict"][t], kk), \
            f"{widths} trail {t}"
        assert np.array_equal(o["impl_lit"][t, :kk], r["impl_lit"][t, :kk]), f"{widths} trail {t}"
        if strategy == "watched":
            assert o["stop"][t] == r["stop"][t], f"{widths} trail {t}"
            assert np.array_equal(o["impl_reason"][t, :kk], r["impl_reason"][t, :kk]), f"{widths} trail {t}"


@pytest.mark.parametrize("strategy", ["watched", "full_scan"])
@pytest.mark.parametrize("k,n,ratio,fmax", SHAPES)
def test_oracle_matches_the_reference_on_fresh_cases(orc, ref, strategy, k, n, ratio, fmax):
    seed = 1000 * k + n
    m = int(round(ratio * n))
    lits, off = orc.gen_random_ksat(seed, n, m, k)
    rng = np.random.default_rng(seed)
    tl, to = make_trails(rng, n, 12, fmax)
    cap = n + 8
    r = ref_run(ref, lits, off, n, tl, to, cap, strategy)
    o = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=cap, strategy=strategy)
    assert r["status"][0] == 0 and r["n_impl"][0] == 0      # the empty trail
    assert r["status"][2] == -2                              # both signs
    assert r["n_impl"].sum() > 0 and (r["status"] == 1).any() and (r["status"] == 0).sum() > 1
    if strategy == "watched":
        compare_bcp(o, r, label=f"k={k} n={n}")
    else:
        # the reference's full-scan entry reports the implied literals and the
        # conflict clause (its sweeps keep no per-implication reason here)
        for t in range(len(to) - 1):
            kk = int(r["n_impl"][t])
            assert (o["status"][t], o["conflict"][t], o["n_impl"][t]) == (r["status"][t], r["conflict"][t], kk), \
                f"k={k} n={n} trail {t}"
            assert np.array_equal(o["impl_lit"][t, :kk], r["impl_lit"][t, :kk]), f"k={k} n={n} trail {t}"
