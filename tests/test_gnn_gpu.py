"""GPU: the learned-seeding kernels against a plain PyTorch fp32 reference of
the same ops.  Inputs and outputs are bf16 (accumulation fp32), so results
are compared with bf16-level tolerances written in each test."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_dev(gpsat, cuda_ok):
    import torch
    return torch, torch.device("cuda:0")


def close(got, want, rtol, atol):
    got, want = got.float(), want.float()
    err = (got - want).abs()
    bound = atol + rtol * want.abs()
    bad = (err > bound).sum().item()
    assert bad == 0, f"{bad} of {err.numel()} elements off; max err {err.max().item():.4g}"


@pytest.mark.parametrize("rows,K,N,ld_extra", [(1000, 64, 192, 0), (300, 64, 64, 0), (128, 128, 64, 0),
                                               (517, 192, 64, 0), (260, 64, 128, 64), (129, 64, 256, 0)])
def test_mm_matches_torch(gpsat, torch_dev, rows, K, N, ld_extra):
    torch, dev = torch_dev
    g = torch.Generator(device="cpu").manual_seed(rows + K + N)
    Xw = torch.randn(rows, K + ld_extra, generator=g).to(dev, torch.bfloat16)
    X = Xw[:, ld_extra:]                               # a column window: row stride K + ld_extra
    B = (torch.randn(N, K, generator=g) / 8).to(dev, torch.bfloat16)
    bias = torch.randn(N, generator=g).to(dev)
    Y = torch.full((rows, N), float("nan"), dtype=torch.bfloat16, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    relu = int(N == 128)
    gpsat.check(gpsat.lib().gpsat_gnn_mm(X.data_ptr(), K + ld_extra, rows, K, B.data_ptr(), K, N, bias.data_ptr(),
                                         relu, Y.data_ptr(), N, err.data_ptr(), None))
    torch.cuda.synchronize()
    assert err.item() == 0
    want = X.float() @ B.float().T + bias
    if relu:
        want = torch.relu(want)
    # bf16 output: relative 2^-8 plus accumulation-order noise
    close(Y, want, rtol=1e-2, atol=2e-2)


@pytest.mark.parametrize("rows,N,ldx_extra,ldy_extra", [(3001, 192, 0, 0), (128, 64, 8, 64), (40000, 128, 128, 64),
                                                      (77, 64, 0, 0)])
def test_wgrad_matches_torch(gpsat, torch_dev, rows, N, ldx_extra, ldy_extra):
    """dW += X^T dY on the tensor cores (rows are the contraction axis, in
    chunks of 128 with a ragged last one), row strides wider than the data."""
    torch, dev = torch_dev
    g = torch.Generator(device="cpu").manual_seed(7)
    Xw = torch.randn(rows, 64 + ldx_extra, generator=g).to(dev, torch.bfloat16)
    Yw = torch.randn(rows, N + ldy_extra, generator=g).to(dev, torch.bfloat16)
    X, dY = Xw[:, :64], Yw[:, :N]
    dW = torch.full((64, N), 0.5, device=dev)          # accumulates into what is there
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    gpsat.check(gpsat.lib().gpsat_gnn_wgrad(X.data_ptr(), 64 + ldx_extra, dY.data_ptr(), N + ldy_extra, rows, N,
                                            dW.data_ptr(), err.data_ptr(), None))
    torch.cuda.synchronize()
    assert err.item() == 0
    want = X.float().T @ dY.float() + 0.5
    # fp32 accumulation of exact bf16 products, summed in another order
    close(dW, want, rtol=1e-4, atol=2e-3 * (rows / 3000) ** 0.5 + 1e-3)


def test_gather_and_split_match_torch(gpsat, torch_dev):
    torch, dev = torch_dev
    from gpupsat_gb300 import learn
    formulas = [gpsat.gen_random_ksat(90 + i, n, int(4.26 * n), 3) for i, n in enumerate((40, 75, 120))]
    nv = [40, 75, 120]
    G = learn.Graph(formulas, nv, dev)
    gen = torch.Generator(device="cpu").manual_seed(3)
    src = torch.randn(G.V, 128, generator=gen).to(dev, torch.bfloat16)
    Z = torch.randn(G.C, 64, generator=gen).to(dev, torch.bfloat16)
    out = torch.empty(G.C, 64, dtype=torch.bfloat16, device=dev)
    L = gpsat.lib()
    gpsat.check(L.gpsat_gnn_gather(G.c_off.data_ptr(), G.c_edges.data_ptr(), G.C, src.data_ptr(),
                                   src.data_ptr() + 128, 128, G.c_scale.data_ptr(), Z.data_ptr(), 64,
                                   out.data_ptr(), 64, 1, None))
    e = G.c_edges.long()
    rowv, pos = e >> 1, (e & 1).bool()
    seg = torch.repeat_interleave(torch.arange(G.C, device=dev), torch.diff(G.c_off))
    msg = torch.where(pos[:, None], src[rowv, :64].float(), src[rowv, 64:].float())
    want = torch.relu(torch.zeros(G.C, 64, device=dev).index_add_(0, seg, msg) * G.c_scale[:, None] + Z.float())
    torch.cuda.synchronize()
    close(out, want, rtol=1e-2, atol=2e-2)
    # split sums over the variable view, each clause row scaled by 1 / its length
    d = torch.randn(G.C, 64, generator=gen).to(dev, torch.bfloat16)
    oP = torch.empty(G.V, 64, dtype=torch.bfloat16, device=dev)
    oN = torch.empty(G.V, 64, dtype=torch.bfloat16, device=dev)
    gpsat.check(L.gpsat_gnn_gather_split(G.v_off.data_ptr(), G.v_edges.data_ptr(), G.V, d.data_ptr(), 64,
                                         G.c_scale.data_ptr(), oP.data_ptr(), oN.data_ptr(), 64, None))
    ds = d.float() * G.c_scale[:, None]
    wP = torch.zeros(G.V, 64, device=dev).index_add_(0, rowv[pos], ds[seg[pos]])
    wN = torch.zeros(G.V, 64, device=dev).index_add_(0, rowv[~pos], ds[seg[~pos]])
    torch.cuda.synchronize()
    close(oP, wP, rtol=1e-2, atol=3e-2)
    close(oN, wN, rtol=1e-2, atol=3e-2)


def torch_reference(torch, net, G, y, w_act, t, w_ph):
    """The network and its losses in plain fp32 autograd on the CPU."""
    from gpupsat_gb300 import learn
    dev = torch.device("cpu")
    P = {k: torch.tensor(v, device=dev, requires_grad=True) for k, v in net.numpy().items()}
    cpu = lambda x: x.detach().to(dev)
    ce, ve = cpu(G.c_edges).long(), cpu(G.v_edges).long()
    c_off, v_off = cpu(G.c_off), cpu(G.v_off)
    c_scale, v_scale = cpu(G.c_scale), cpu(G.v_scale)
    y, w_act, t, w_ph = cpu(y), cpu(w_act), cpu(t), cpu(w_ph)
    c_seg = torch.repeat_interleave(torch.arange(G.C), torch.diff(c_off))
    v_seg = torch.repeat_interleave(torch.arange(G.V), torch.diff(v_off))
    F = cpu(G.feat)[:G.V].float()
    Hv = torch.relu(F @ P["Win"] + P["bin"])
    Hc = P["hc0"].expand(G.C, 64)
    for l in range(learn.LAYERS):
        A3 = Hv @ P[f"Wv3_{l}"] + P[f"bias3_{l}"]
        Zc = Hc @ P[f"Wc_{l}"] + P[f"bc_{l}"]
        r, s = ce >> 1, (ce & 1).bool()
        msg = torch.where(s[:, None], A3[r, :64], A3[r, 64:128])
        Hc = torch.relu(torch.zeros(G.C, 64).index_add(0, c_seg, msg) * c_scale[:, None] + Zc)
        Bm = Hc @ P[f"U_{l}"]
        r, s = ve >> 1, (ve & 1).bool()
        msg = torch.where(s[:, None], Bm[r, :64], Bm[r, 64:])
        Hv = torch.relu(torch.zeros(G.V, 64).index_add(0, v_seg, msg) * v_scale[:, None] + A3[:, 128:])
    h = P["head"]
    score = Hv @ h[:64] + h[128]
    phase = Hv @ h[64:128] + h[129]
    ps, pp = torch.sigmoid(score), torch.sigmoid(phase)
    la = (((ps - y) ** 2) * w_act).sum()
    lp = (-(t * torch.log(pp.clamp_min(1e-12)) + (1 - t) * torch.log((1 - pp).clamp_min(1e-12))) * w_ph).sum()
    (la + lp).backward()
    return float(la.detach()), float(lp.detach()), {k: v.grad.detach().cpu().numpy() for k, v in P.items()}, \
        score.detach()


def test_forward_backward_match_autograd(gpsat, torch_dev):
    torch, dev = torch_dev
    from gpupsat_gb300 import learn
    ns = [60, 90, 150, 33]
    formulas = [gpsat.gen_random_ksat(300 + i, n, int(round(4.26 * n)), 3) for i, n in enumerate(ns)]
    net = learn.SeedNet(dev, seed=5)
    G = learn.Graph(formulas, ns, dev)
    rng = np.random.default_rng(1)
    y = torch.tensor(rng.random(G.V), dtype=torch.float32, device=dev)
    t = torch.tensor(rng.random(G.V) < 0.5, dtype=torch.float32, device=dev)
    w_act = torch.full((G.V,), 1.0 / G.V, device=dev)
    w_ph = torch.full((G.V,), 0.5 / G.V, device=dev)
    ps = learn.Pass(net, G)
    ps.forward()
    score = torch.empty(G.V, device=dev)
    ps.heads(score, None)
    loss = torch.zeros(2, device=dev)
    ps.loss_backward(y, w_act, t, w_ph, loss)
    torch.cuda.synchronize()
    assert ps.err.item() == 0
    la, lp, grads, want_score = torch_reference(torch, net, G, y, w_act, t, w_ph)
    # forward: bf16 activations through 3 layers
    close(score.cpu(), want_score, rtol=5e-2, atol=5e-2)
    got_loss = loss.cpu().numpy()
    assert abs(got_loss[0] - la) <= 0.03 * abs(la) + 1e-4 and abs(got_loss[1] - lp) <= 0.03 * abs(lp) + 1e-4
    # backward: every parameter block's gradient points the same way and has the same size
    flat = net.g.cpu().numpy()
    for k, (o, shp) in net.index.items():
        got = flat[o:o + int(np.prod(shp))]
        want = grads[k].reshape(-1)
        if k.startswith("bias3"):
            got, want = got[128:], want[128:]        # the A part of this bias is fixed at zero
        nw = np.linalg.norm(want)
        if nw < 1e-8:
            assert np.linalg.norm(got) < 1e-5, k
            continue
        cos = float(got @ want / (np.linalg.norm(got) * nw + 1e-30))
        assert cos > 0.98, f"{k}: cosine {cos:.4f}"
        assert 0.9 < np.linalg.norm(got) / nw < 1.1, f"{k}: norm ratio {np.linalg.norm(got) / nw:.3f}"


def test_training_lowers_the_loss(gpsat, torch_dev):
    torch, dev = torch_dev
    from gpupsat_gb300 import learn
    ns = list(range(60, 140, 5))
    formulas = [gpsat.gen_random_ksat(700 + i, n, int(round(4.26 * n)), 3) for i, n in enumerate(ns)]
    y, t, has_phase, out = learn.participation_targets(formulas, ns, conflict_budget=2000)
    assert (out["verdict"] != 0).any()
    net = learn.SeedNet(dev, seed=1)
    losses = [sum(learn.train_step(net, formulas, ns, y, t, has_phase, lr=3e-3)) for _ in range(80)]
    # the phase term of random 3-SAT stays near log 2; the activity term falls
    assert np.mean(losses[-5:]) < 0.9 * np.mean(losses[:5]), losses[::10]
    score, phase = learn.predict(net, formulas, ns)
    act, ph = learn.seeds_from(score, phase)
    b = gpsat.Batch(formulas, ns)
    b.set_seeds(act, ph)
    res = b.solve()
    assert (res["model_ok"][res["verdict"] == gpsat.SAT] == 1).all()


def test_learned_seeding_against_plain_vsids(gpsat, torch_dev):
    """What the trained network gains over the plain solver: trained (every
    forward and backward step in the library's kernels) on labels the plain
    solver logs on 2,048 random k-SAT training formulas (k in {3, 4, 5} near
    threshold, n in [100, 400]), then 1,024 held-out instances of the batched
    workload's distribution (random 3-SAT, n in [50, 250], ratio 4.26; formula
    seeds the workload does not use) are solved plain and seeded.  Verdicts
    agree wherever both decide, every model checks, and the seeded arm needs
    fewer conflicts at the median."""
    torch, dev = torch_dev
    from gpupsat_gb300 import learn
    torch.manual_seed(0)
    net = learn.SeedNet(dev, seed=0)
    learn.train(net, learn.training_set(2048, seed=0), epochs=3, conflict_budget=20000, log=None)
    rng = np.random.default_rng(29)
    ns = [int(n) for n in rng.integers(50, 251, size=1024)]
    formulas = [gpsat.gen_random_ksat(90000 + i, n, int(round(4.26 * n)), 3) for i, n in enumerate(ns)]
    opts = gpsat.solve_options(conflict_budget=100000)
    plain = gpsat.Batch(formulas, ns).solve(opts)
    score, phase = learn.predict(net, formulas, ns)
    b = gpsat.Batch(formulas, ns)
    b.set_seeds(*learn.seeds_from(score, phase))
    seeded = b.solve(opts)
    vp, vs = plain["verdict"], seeded["verdict"]
    both = (vp != 0) & (vs != 0)
    assert (vp[both] == vs[both]).all()
    assert (seeded["model_ok"][vs == gpsat.SAT] == 1).all()
    cp, cs = plain["stats"][:, 0], seeded["stats"][:, 0]
    mp, ms = np.median(cp), np.median(cs)
    print(f"median conflicts: plain {mp:.0f}, seeded {ms:.0f} ({100 * (1 - ms / mp):+.1f}% fewer); "
          f"mean {cp.mean():.0f} vs {cs.mean():.0f}; decided: plain {int((vp != 0).sum())}, "
          f"seeded {int((vs != 0).sum())}; seeded fewer on {(cs < cp).mean():.2%} of instances")
    assert ms < mp
