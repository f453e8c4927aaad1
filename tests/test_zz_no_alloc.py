"""GPU: the allocation-free BCP entry point (gpsat_bcp_run_static) gives the
same outputs as gpsat_bcp_run_device on two calls in a row, rejects a
formula whose per-trail state does not fit its fixed scratch, and refuses a
formula that is not on the device yet.  Collected last, so it also runs after
every other GPU test in the same process; it needs nothing they leave."""
import numpy as np
import pytest

from conftest import compare_bcp

pytestmark = pytest.mark.gpu


def device_out(torch, T, cap, dev, fill=-7):
    return dict(status=torch.full((T,), fill, dtype=torch.int32, device=dev),
                conflict=torch.full((T,), fill, dtype=torch.int32, device=dev),
                stop=torch.full((T,), fill, dtype=torch.int32, device=dev),
                n_impl=torch.full((T,), fill, dtype=torch.int64, device=dev),
                impl_lit=torch.zeros(T, cap, dtype=torch.int32, device=dev),
                impl_reason=torch.zeros(T, cap, dtype=torch.int32, device=dev),
                counters=torch.zeros(T, 6, dtype=torch.int64, device=dev))


def to_host(out):
    return {k: v.cpu().numpy() for k, v in out.items()}


def test_static_entry_matches_device_entry_twice(gpsat, cuda_ok):
    import torch
    dev = torch.device("cuda:0")
    cap = 512
    n = 5000
    lits, off = gpsat.gen_random_ksat(31, n, 21000, 3)
    f = gpsat.Formula(lits, off, n)
    b = gpsat.BCPBatch(f, impl_cap=cap)          # uploads the formula
    s = torch.cuda.Stream()
    # two calls in a row with different trail sets (the second must not see
    # the first one's state), each against the allocating entry point
    for seed, T in ((32, 300), (33, 173)):
        tl, to = gpsat.gen_trails(seed, n, T, 0.01, 0.08)
        d_tl, d_to = torch.from_numpy(tl).to(dev), torch.from_numpy(to).to(dev)
        want = device_out(torch, T, cap, dev)
        got = device_out(torch, T, cap, dev, fill=-9)
        with torch.cuda.stream(s):
            b.run_device(d_tl, d_to, want, stream=s.cuda_stream)
            gpsat.bcp_run_static(f, d_tl, d_to, got, impl_cap=cap, stream=s.cuda_stream)
        s.synchronize()
        w, g = to_host(want), to_host(got)
        compare_bcp(g, w, label=f"static entry, {T} trails")
        assert np.array_equal(g["counters"], w["counters"])
        assert (g["status"] == 1).any() and (g["status"] == 0).any()


def test_static_entry_after_another_formula(gpsat, cuda_ok):
    # a larger formula, then a smaller one: the layout changes between calls
    import torch
    dev = torch.device("cuda:0")
    cap = 256
    for n, m, seed in ((20000, 84000, 41), (700, 2940, 42)):
        lits, off = gpsat.gen_random_ksat(seed, n, m, 3)
        f = gpsat.Formula(lits, off, n)
        b = gpsat.BCPBatch(f, impl_cap=cap)
        tl, to = gpsat.gen_trails(seed + 1, n, 128, 0.01, 0.05)
        d_tl, d_to = torch.from_numpy(tl).to(dev), torch.from_numpy(to).to(dev)
        got = device_out(torch, 128, cap, dev)
        gpsat.bcp_run_static(f, d_tl, d_to, got, impl_cap=cap)
        torch.cuda.synchronize()
        compare_bcp(to_host(got), b.run_host(tl, to), label=f"static entry n={n}")


def test_static_entry_rejects_state_beyond_its_scratch(gpsat, cuda_ok):
    import torch
    dev = torch.device("cuda:0")
    n = 1000
    lits, off = gpsat.gen_random_ksat(51, n, 4200, 3)
    f = gpsat.Formula(lits, off, n)
    gpsat.BCPBatch(f, impl_cap=64)
    tl, to = gpsat.gen_trails(52, n, 4, 0.01, 0.05)
    d_tl, d_to = torch.from_numpy(tl).to(dev), torch.from_numpy(to).to(dev)
    # 2^24 watch moves of room for one trail is far beyond the 64 MiB array;
    # the output buffers match impl_cap, so even a call that got through
    # would stay inside them
    out = device_out(torch, 4, 1, dev)
    with pytest.raises(gpsat.GpsatError) as e:
        gpsat.bcp_run_static(f, d_tl, d_to, out, impl_cap=1, arena_cap=1 << 24)
    assert e.value.code == -6 and "static scratch holds 67108864 bytes" in str(e.value)  # GPSAT_ERR_CAPACITY
    torch.cuda.synchronize()
    assert (out["status"] == -7).all()                # nothing was launched


def test_static_entry_needs_a_resident_formula(gpsat, cuda_ok):
    import torch
    dev = torch.device("cuda:0")
    lits, off = gpsat.gen_random_ksat(61, 300, 1260, 3)
    f = gpsat.Formula(lits, off, 300)                  # never uploaded
    tl, to = gpsat.gen_trails(62, 300, 2, 0.01, 0.05)
    out = device_out(torch, 2, 64, dev)
    with pytest.raises(gpsat.GpsatError) as e:
        gpsat.bcp_run_static(f, torch.from_numpy(tl).to(dev), torch.from_numpy(to).to(dev), out, impl_cap=64)
    assert e.value.code == -9                           # GPSAT_ERR_STATE


def test_static_entry_replays_inside_a_cuda_graph(gpsat, cuda_ok):
    """The allocation-free entry captured once into a CUDA graph and replayed:
    each replay re-reads the (rewritten) trail buffers and matches the
    allocating entry point on the same trails."""
    import torch
    dev = torch.device("cuda:0")
    cap = 256
    n, T = 3000, 96
    lits, off = gpsat.gen_random_ksat(71, n, 12600, 3)
    f = gpsat.Formula(lits, off, n)
    b = gpsat.BCPBatch(f, impl_cap=cap)
    sets = [gpsat.gen_trails(72 + k, n, T, 0.02, 0.02) for k in range(3)]   # equal lengths: fixed offsets
    assert all(np.array_equal(s[1], sets[0][1]) for s in sets)
    d_tl = torch.from_numpy(sets[0][0]).to(dev)
    d_to = torch.from_numpy(sets[0][1]).to(dev)
    got = device_out(torch, T, cap, dev)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):   # the first call on the device looks its array up: before any capture
        gpsat.bcp_run_static(f, d_tl, d_to, got, impl_cap=cap, stream=s.cuda_stream)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        gpsat.bcp_run_static(f, d_tl, d_to, got, impl_cap=cap, stream=s.cuda_stream)
    for tl, to in sets[1:]:
        d_tl.copy_(torch.from_numpy(tl))
        g.replay()
        torch.cuda.synchronize()
        want = b.run_host(tl, to)
        compare_bcp(to_host(got), want, label="graph replay")
        assert np.array_equal(to_host(got)["counters"], want["counters"])
