"""GPU: the sm_103a reference-order BCP kernel, called through the C ABI, is
bit-exact against the reference's own outputs (golden vectors) and against
the oracle on seeded inputs, including edge cases and the full-size
benchmark shape (n = 1e6, m = 4.2e6, 4096 trails)."""
import numpy as np
import pytest

from conftest import compare_bcp

pytestmark = pytest.mark.gpu


def run_both(gpsat, orc, lits, off, n, tl, to, impl_cap=4096, max_slots=0, arena_cap=0, threads=8):
    f = gpsat.Formula(lits, off, n)
    b = gpsat.BCPBatch(f, max_slots=max_slots, impl_cap=impl_cap, arena_cap=arena_cap)
    g = b.run_host(tl, to)
    o = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=impl_cap, threads=threads)
    return g, o


def test_bcp_matches_reference_golden(gpsat, cuda_ok, bcp_golden):
    for ci, c in enumerate(bcp_golden):
        n = int(c["n"][0])
        f = gpsat.Formula(c["lits"], c["off"], n)
        b = gpsat.BCPBatch(f, impl_cap=max(64, n))
        g = b.run_host(c["tl"], c["to"])
        compare_bcp(g, c, label=f"golden case {ci}")


@pytest.mark.parametrize("n,ratio,k,T,fmin,fmax,seed", [
    (100, 4.26, 3, 200, 0.01, 0.30, 1),
    (2000, 4.2, 3, 512, 0.01, 0.05, 2),
    (20000, 4.2, 3, 512, 0.01, 0.05, 3),
    (500, 9.9, 4, 256, 0.05, 0.40, 4),
    (300, 21.0, 5, 256, 0.05, 0.50, 5),
    # 524,300 variables: the trail-application kernel's second shared-memory
    # chunk of assignment words holds one word (its variables 524,288 onward)
    (524300, 4.2, 3, 32, 0.002, 0.01, 6),
])
def test_bcp_matches_oracle_random(gpsat, orc, cuda_ok, n, ratio, k, T, fmin, fmax, seed):
    m = int(round(ratio * n))
    lits, off = gpsat.gen_random_ksat(seed, n, m, k)
    tl, to = gpsat.gen_trails(seed + 77, n, T, fmin, fmax)
    g, o = run_both(gpsat, orc, lits, off, n, tl, to, impl_cap=n)
    compare_bcp(g, o, label=f"n={n} k={k}")
    bad = np.nonzero((g["counters"] != o["counters"]).any(1))[0]
    assert len(bad) == 0, (f"counters differ on {len(bad)} trails, first {bad[:5].tolist()}: gpu "
                           f"{g['counters'][bad[:3]].tolist()} oracle {o['counters'][bad[:3]].tolist()} "
                           f"status {g['status'][bad[:3]].tolist()} n_impl {g['n_impl'][bad[:3]].tolist()} "
                           f"len {(to[bad[:3] + 1] - to[bad[:3]]).tolist()}")
    assert (g["status"] == 1).any() and (g["status"] == 0).any() or T < 300


def test_bcp_edge_cases(gpsat, orc, cuda_ok):
    n = 200
    lits, off = gpsat.gen_random_ksat(8, n, 852, 3)
    trails = [
        [],                        # empty trail
        [5],                       # one literal
        [3, -7, 3, 11],            # repeated literal, same sign: propagated twice
        [4, 9, -4],                # a variable both ways: rejected
        [1, 2, 250],               # variable out of range: rejected
        list(range(1, n + 1)),     # every variable
        [-v for v in range(n, 0, -1)],
    ]
    to = np.zeros(len(trails) + 1, np.int64)
    to[1:] = np.cumsum([len(t) for t in trails])
    tl = np.array([x for t in trails for x in t], np.int32)
    f = gpsat.Formula(lits, off, n)
    g = gpsat.BCPBatch(f, impl_cap=n).run_host(tl, to)
    assert list(g["status"][3:5]) == [-2, -2]
    ok = [0, 1, 2, 5, 6]
    o = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=n)
    compare_bcp(g, o, label="edge")
    assert g["n_impl"][0] == 0 and g["status"][0] == 0 and g["counters"][0, 0] == 0
    assert all(g["counters"][t, 5] == len(trails[t]) for t in ok)


def test_bcp_bad_trail_offsets_are_refused(gpsat, cuda_ok):
    """Host entry: offsets that go back, start below 0 or run past the literals
    are refused before anything is copied; the handle still runs after."""
    lits, off = gpsat.gen_random_ksat(9, 100, 426, 3)
    b = gpsat.BCPBatch(gpsat.Formula(lits, off, 100), impl_cap=100)
    tl = np.array([1, -2, 3, 4, -5, 6], np.int32)
    for to in ([0, 4, 2, 6], [-1, 2, 6]):
        with pytest.raises(gpsat.GpsatError):
            b.run_host(tl, np.array(to, np.int64))
    with pytest.raises(ValueError):
        b.run_host(tl, np.array([0, 2, 9], np.int64))
    g = b.run_host(tl, np.array([0, 2, 6], np.int64))
    assert set(g["status"]) <= {0, 1}


def test_bcp_slot_reuse_and_epoch_wrap(gpsat, orc, cuda_ok):
    # one slot serves 400 trails: it runs past its 255-trail epoch range and
    # wipes its list heads and clause states once
    n = 1000
    lits, off = gpsat.gen_random_ksat(12, n, 4200, 3)
    tl, to = gpsat.gen_trails(13, n, 400, 0.01, 0.10)
    g, o = run_both(gpsat, orc, lits, off, n, tl, to, impl_cap=n, max_slots=1)
    compare_bcp(g, o, label="slot reuse")


def test_bcp_active_slots_do_not_change_outputs(gpsat, orc, cuda_ok):
    # fewer trails in flight than allocated slots (and the ordering kernels
    # that come with more trails than active slots): same outputs
    n = 3000
    lits, off = gpsat.gen_random_ksat(16, n, 12600, 3)
    tl, to = gpsat.gen_trails(17, n, 200, 0.01, 0.08)
    f = gpsat.Formula(lits, off, n)
    b = gpsat.BCPBatch(f, max_slots=64, impl_cap=n)
    full = b.run_host(tl, to)
    for k in (5, 1, 0):
        b.set_active_slots(k)
        compare_bcp(b.run_host(tl, to), full, label=f"active slots {k}")
    for bad in (-1, 65):
        with pytest.raises(gpsat.GpsatError) as e:
            b.set_active_slots(bad)
        assert e.value.code == -1
    o = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=n)
    compare_bcp(full, o, label="oracle")


def test_bcp_capacity_overflow_is_reported(gpsat, orc, cuda_ok):
    n = 2000
    lits, off = gpsat.gen_random_ksat(14, n, 8400, 3)
    tl, to = gpsat.gen_trails(15, n, 64, 0.02, 0.10)
    g, o = run_both(gpsat, orc, lits, off, n, tl, to, impl_cap=3)
    compare_bcp(g, o, label="implication cap")
    assert (g["status"] == -1).any()
    f = gpsat.Formula(lits, off, n)
    g2 = gpsat.BCPBatch(f, impl_cap=n, arena_cap=2).run_host(tl, to)
    over = g2["status"] == -1
    assert over.mean() > 0.8
    # trails that finished inside the tiny move arena are still exact
    o2 = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=n)
    compare_bcp({k: v[~over] for k, v in g2.items() if v is not None}, o2, trails=list(np.nonzero(~over)[0]),
                label="arena cap")


def test_bcp_device_entry_matches_host_entry(gpsat, cuda_ok):
    import torch
    n = 5000
    lits, off = gpsat.gen_random_ksat(21, n, 21000, 3)
    tl, to = gpsat.gen_trails(22, n, 300, 0.01, 0.05)
    f = gpsat.Formula(lits, off, n)
    b = gpsat.BCPBatch(f, impl_cap=512)
    h = b.run_host(tl, to)
    dev = torch.device("cuda:0")
    T = len(to) - 1
    out = dict(status=torch.empty(T, dtype=torch.int32, device=dev),
               conflict=torch.empty(T, dtype=torch.int32, device=dev),
               stop=torch.empty(T, dtype=torch.int32, device=dev),
               n_impl=torch.empty(T, dtype=torch.int64, device=dev),
               impl_lit=torch.zeros(T, 512, dtype=torch.int32, device=dev),
               impl_reason=torch.zeros(T, 512, dtype=torch.int32, device=dev),
               counters=torch.zeros(T, 6, dtype=torch.int64, device=dev))
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b.run_device(torch.from_numpy(tl).to(dev), torch.from_numpy(to).to(dev), out, stream=s.cuda_stream)
    s.synchronize()
    d = {k: v.cpu().numpy() for k, v in out.items()}
    compare_bcp(d, h, label="device entry")
    assert np.array_equal(d["counters"], h["counters"])


def test_bcp_pinned_host_buffers_in_place(gpsat, cuda_ok):
    # page-locked inputs and outputs are used in place by the kernel: same
    # results as the staged (pageable) path
    import torch
    n = 5000
    lits, off = gpsat.gen_random_ksat(23, n, 21000, 3)
    tl, to = gpsat.gen_trails(24, n, 300, 0.01, 0.05)
    b = gpsat.BCPBatch(gpsat.Formula(lits, off, n), impl_cap=512)
    h = b.run_host(tl, to)
    tdt = {np.int32: torch.int32, np.int64: torch.int64}
    pinned = lambda shape, dt: torch.zeros(shape, dtype=tdt[dt], pin_memory=True).numpy()
    p_tl, p_to = pinned(tl.shape, np.int32), pinned(to.shape, np.int64)
    p_tl[:] = tl
    p_to[:] = to
    out = b.host_outputs(len(to) - 1, counters=True, alloc=pinned)
    for _ in range(2):
        p = b.run_host(p_tl, p_to, out=out)
        compare_bcp(p, h, label="pinned in place")
        assert np.array_equal(p["counters"], h["counters"])


def test_bcp_full_size_benchmark_shape(gpsat, orc, cuda_ok):
    """n=1e6, m=4.2e6, 4096 trails at 1-5%: a seeded sample of 96 trails is
    compared bit-exactly with the oracle; every trail's outputs are checked for
    size-independent properties (each reason clause is unit for its literal
    under the trail and earlier implications; a conflict clause is all false)."""
    n, m, T = 1_000_000, 4_200_000, 4096
    lits, off = gpsat.gen_random_ksat(2024, n, m, 3)
    tl, to = gpsat.gen_trails(7, n, T, 0.01, 0.05)
    f = gpsat.Formula(lits, off, n)
    g = gpsat.BCPBatch(f, impl_cap=4096).run_host(tl, to)
    assert set(np.unique(g["status"])) <= {0, 1}
    rng = np.random.default_rng(5)
    sample = np.sort(rng.choice(T, 96, replace=False))
    sub_to = np.zeros(len(sample) + 1, np.int64)
    sub_to[1:] = np.cumsum(to[sample + 1] - to[sample])
    sub_tl = np.concatenate([tl[to[t]:to[t + 1]] for t in sample])
    o = orc.BCPOracle(lits, off, n).run(sub_tl, sub_to, impl_cap=4096, threads=16)
    compare_bcp(o, g, trails=list(sample), label="full size")
    cl = lits.reshape(-1, 3)
    BIG = np.int64(1) << 40
    for t in range(0, T, 4):
        tr = tl[to[t]:to[t + 1]]
        k = int(g["n_impl"][t])
        imp = g["impl_lit"][t, :k]
        sgn = np.zeros(n + 1, np.int8)
        pos = np.full(n + 1, BIG, np.int64)   # -1: trail, j: j-th implication
        sgn[np.abs(tr)] = np.sign(tr)
        pos[np.abs(tr)] = -1
        assert (pos[np.abs(imp)] == BIG).all(), f"trail {t}: implied an assigned variable"
        sgn[np.abs(imp)] = np.sign(imp)
        pos[np.abs(imp)] = np.arange(k)
        if k:
            rc = cl[g["impl_reason"][t, :k]]                       # k x 3
            is_unit = rc == imp[:, None]
            assert is_unit.sum(1).min() == 1, f"trail {t}: implied literal missing from its reason"
            other = ~is_unit
            false_before = (sgn[np.abs(rc)] == -np.sign(rc)) & (pos[np.abs(rc)] < np.arange(k)[:, None])
            assert (false_before | ~other).all(), f"trail {t}: a reason clause is not unit"
        if g["status"][t] == 1:
            c = cl[g["conflict"][t]]
            assert (sgn[np.abs(c)] == -np.sign(c)).all(), f"trail {t}: conflict clause not false"


def test_bcp_window_widths_agree(gpsat, orc, cuda_ok):
    """The kernel at 64, 128 and 256 watch entries per round (2, 4 and 8 warps
    per trail): the same outputs and counters, equal to the oracle's; the
    autotuner picks one of them."""
    import torch
    n = 20000
    lits, off = gpsat.gen_random_ksat(44, n, 84000, 3)
    tl, to = gpsat.gen_trails(45, n, 300, 0.01, 0.05)
    b = gpsat.BCPBatch(gpsat.Formula(lits, off, n), impl_cap=2048)
    o = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=2048, threads=8)
    for w in (64, 256, 128):
        b.set_window(w)
        assert b.window_slots(w) >= 1
        g = b.run_host(tl, to)
        compare_bcp(g, o, label=f"window {w}")
        assert np.array_equal(g["counters"], o["counters"])
    with pytest.raises(gpsat.GpsatError):
        b.set_window(96)
    dev = torch.device("cuda:0")
    T = len(to) - 1
    out = dict(status=torch.empty(T, dtype=torch.int32, device=dev),
               conflict=torch.empty(T, dtype=torch.int32, device=dev),
               stop=torch.empty(T, dtype=torch.int32, device=dev),
               n_impl=torch.empty(T, dtype=torch.int64, device=dev),
               impl_lit=torch.empty(T, 2048, dtype=torch.int32, device=dev),
               impl_reason=torch.empty(T, 2048, dtype=torch.int32, device=dev),
               counters=torch.empty(T, 6, dtype=torch.int64, device=dev))
    s = torch.cuda.Stream()
    times = b.tune(torch.from_numpy(tl).to(dev), torch.from_numpy(to).to(dev), out, s.cuda_stream)
    assert b.window in (64, 128, 256) and (b.window, b.active, b.pivot) in times
    s.synchronize()
    compare_bcp({k: v.cpu().numpy() for k, v in out.items()}, o, label="after tuning")


def test_bcp_order_pivot_does_not_change_outputs(gpsat, orc, cuda_ok):
    """More trails than slots, so the processing order applies: trails nearest
    each pivot first (0 = shortest first) give the same outputs as the oracle;
    a negative pivot is refused."""
    n = 5000
    lits, off = gpsat.gen_random_ksat(46, n, 21000, 3)
    tl, to = gpsat.gen_trails(47, n, 200, 0.005, 0.08)
    b = gpsat.BCPBatch(gpsat.Formula(lits, off, n), impl_cap=2048)
    b.set_active_slots(8)
    o = orc.BCPOracle(lits, off, n).run(tl, to, impl_cap=2048, threads=8)
    lens = np.diff(to)
    for p in (0, int(np.median(lens)), int(lens.max()) + 1000, 1 << 40):
        b.set_order_pivot(p)
        g = b.run_host(tl, to)
        compare_bcp(g, o, label=f"pivot {p}")
        assert np.array_equal(g["counters"], o["counters"])
    with pytest.raises(gpsat.GpsatError):
        b.set_order_pivot(-1)
