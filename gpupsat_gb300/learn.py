"""Learned seeding for the device CDCL solver.

A 3-layer, 64-wide message-passing network over the variable-clause graph
predicts, per variable, (1) how often it takes part in conflicts and (2) its
value in a model.  The predictions seed the solver's VSIDS activities and
saved phases (Batch.set_seeds) and rank the JobChooser's split variables
(jobs.cube_jobs(scores=...)).  The reference has no learned component; what
it seeds are the reference's DecisionStrategy (SATSolver/DecisionMaker.cu,
DecisionStrategy/VSIDS.cu) and JobChooser (JobsManager/VariableChooser.cu)
inputs.

Every forward and backward step runs in libgpsat's hand-written kernels
(gnn.cu: tcgen05 matrix products, message sums, heads, Adam); torch only
allocates device memory.  The training labels come from the solver itself:
per-variable conflict participation and learnt-clause occurrence counts
logged during budgeted solves (Batch.solve(participation=2)) and the models
of satisfiable instances.

Variable features F_v (64 wide, zero padded): log(1 + occurrences) by
polarity, log(1 + number of clauses of length k holding v) for k = 3..7
(longer clauses count as 7), the variable's community id / 40 (planted
instances; 0 otherwise) and a constant 1.

Network, per layer l = 1..3 (H_v^0 = relu(F_v Win + bin), H_c^0 = hc0):
    [A+ | A- | Zv] = H_v^{l-1} Wv3_l + bias3_l          Wv3_l = [W+ | W- | Wv]
    H_c^l = relu(mean_{(v,s) in c} A_s[v] + H_c^{l-1} Wc_l + bc_l)
    [B+ | B-] = H_c^l U_l                                U_l = [U+ | U-]
    H_v^l = relu(mean_{c ∋ (v,s)} B_s[c] + Zv)
    score_v = H_v^3 . ws + bs,  phase_v = H_v^3 . wp + bp
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import check, lib

D = 64          # hidden width
LAYERS = 3


def _p(t):
    return None if t is None else t.data_ptr()


def _off(t, elems):
    """Address of a tensor plus an element offset (bf16 = 2 bytes)."""
    return t.data_ptr() + 2 * elems


# ---------------------------------------------------------------- graphs
class Graph:
    """The variable-clause graph of a batch of formulas on the device.

    Variables and clauses of all formulas are numbered globally (formula f's
    variable v is row var_base[f] + v - 1).  Two CSR views of the edges:
    by clause (its literals: variable row, sign) and by variable (the
    clauses it occurs in: clause row, sign); an edge is (row << 1) | positive.
    """

    def __init__(self, formulas, n_vars, device, communities=None):
        import torch
        n_vars = np.asarray(n_vars, np.int64)
        self.var_base = np.zeros(len(formulas) + 1, np.int64)
        self.var_base[1:] = np.cumsum(n_vars)
        lit_parts, off_parts, cbase = [], [], [0]
        for (lits, off), vb in zip(formulas, self.var_base[:-1]):
            lits = np.asarray(lits, np.int64)
            lit_parts.append(np.sign(lits) * (np.abs(lits) + vb))
            off_parts.append(np.asarray(off, np.int64)[1:] - np.asarray(off, np.int64)[0])
            cbase.append(cbase[-1] + len(off) - 1)
        self.clause_base = np.asarray(cbase, np.int64)
        glits = np.concatenate(lit_parts) if lit_parts else np.zeros(0, np.int64)
        lens = np.concatenate([np.diff(np.concatenate([[0], o])) for o in off_parts]) if off_parts else np.zeros(0)
        self.V = int(self.var_base[-1])
        self.C = int(self.clause_base[-1])
        coff = np.zeros(self.C + 1, np.int64)
        coff[1:] = np.cumsum(lens)
        vrow = np.abs(glits) - 1
        pos = (glits > 0).astype(np.int64)
        cedges = (vrow << 1) | pos
        crow = np.repeat(np.arange(self.C, dtype=np.int64), lens.astype(np.int64))
        order = np.argsort(vrow, kind="stable")
        voff = np.zeros(self.V + 1, np.int64)
        voff[1:] = np.cumsum(np.bincount(vrow, minlength=self.V))
        vedges = (crow[order] << 1) | pos[order]
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dt)).to(device)
        self.c_off, self.c_edges = t(coff, np.int64), t(cedges, np.int32)
        self.v_off, self.v_edges = t(voff, np.int64), t(vedges, np.int32)
        # message means: 1 / degree per clause and per variable (1 for degree 0)
        self.c_scale = t(1.0 / np.maximum(np.diff(coff), 1), np.float32)
        self.v_scale = t(1.0 / np.maximum(np.diff(voff), 1), np.float32)
        # variable features
        F = np.zeros((max(self.V, 1), D), np.float32)
        F[:self.V, 0] = np.log1p(np.bincount(vrow[pos == 1], minlength=self.V))
        F[:self.V, 1] = np.log1p(np.bincount(vrow[pos == 0], minlength=self.V))
        clen = np.minimum(np.maximum(lens.astype(np.int64), 3), 7)[crow] if len(crow) else np.zeros(0, np.int64)
        for k in range(3, 8):
            F[:self.V, 2 + k - 3] = np.log1p(np.bincount(vrow[clen == k], minlength=self.V))
        if communities is not None:
            F[:self.V, 7] = np.concatenate([np.asarray(c, np.float32) for c in communities]) / 40.0
        F[:self.V, 8] = 1.0
        self.feat_host = F[:self.V]
        self.feat = torch.from_numpy(F).to(device=device, dtype=torch.bfloat16)
        self.E = len(glits)
        self.device = device


# ---------------------------------------------------------------- parameters
class SeedNet:
    """Parameters (fp32 master copy in one flat buffer, for Adam) and their
    bf16 operand copies for the matrix-product kernel."""

    def __init__(self, device, seed: int = 0):
        import torch
        self.device = device
        rng = np.random.default_rng(seed)
        shapes = [("Win", (D, D)), ("bin", (D,)), ("hc0", (D,))]
        for l in range(LAYERS):
            shapes += [(f"Wv3_{l}", (D, 3 * D)), (f"bias3_{l}", (3 * D,)), (f"Wc_{l}", (D, D)), (f"bc_{l}", (D,)),
                       (f"U_{l}", (D, 2 * D))]
        shapes += [("head", (2 * D + 2,))]
        self.shapes = shapes
        sizes = [int(np.prod(s)) for _, s in shapes]
        self.n = sum(sizes)
        flat = np.zeros(self.n, np.float32)
        self.index = {}
        o = 0
        for (name, shp), sz in zip(shapes, sizes):
            self.index[name] = (o, shp)
            if name.startswith(("Wv3", "Wc", "U", "Win")):
                flat[o:o + sz] = rng.normal(0.0, 1.0 / math.sqrt(D), sz)
            elif name == "hc0":
                flat[o:o + sz] = rng.normal(0.0, 1.0, sz)
            elif name == "head":
                flat[o:o + 2 * D] = rng.normal(0.0, 1.0 / math.sqrt(D), 2 * D)
            o += sz
        f32 = dict(dtype=torch.float32, device=device)
        self.p = torch.from_numpy(flat).to(device)
        self.g = torch.zeros(self.n, **f32)
        self.m = torch.zeros(self.n, **f32)
        self.v = torch.zeros(self.n, **f32)
        self.step = 0
        bf = dict(dtype=torch.bfloat16, device=device)
        # operands: forward B = W^T; backward B = W, with [U_l | Wc_{l+1}] side by side
        self.fwd_v = [torch.empty(3 * D, D, **bf) for _ in range(LAYERS)]
        self.fwd_c = [torch.empty(D, D, **bf) for _ in range(LAYERS)]
        self.fwd_u = [torch.empty(2 * D, D, **bf) for _ in range(LAYERS)]
        self.bwd_v = [torch.empty(D, 3 * D, **bf) for _ in range(LAYERS)]
        self.bwd_c = [torch.empty(D, 3 * D, **bf) for _ in range(LAYERS)]   # [U_l | Wc_{l+1}] (last: U only)
        self.bwd_c1 = torch.empty(D, D, **bf)                                 # Wc_0 alone
        self.fwd_in = torch.empty(D, D, **bf)
        self.pack()

    def ptr(self, name, grad=False):
        o, _ = self.index[name]
        return (self.g if grad else self.p).data_ptr() + 4 * o

    def numpy(self) -> dict:
        flat = self.p.cpu().numpy()
        return {k: flat[o:o + int(np.prod(s))].reshape(s).copy() for k, (o, s) in self.index.items()}

    def load(self, params: dict) -> None:
        import torch
        flat = self.p.cpu().numpy()
        for k, (o, s) in self.index.items():
            flat[o:o + int(np.prod(s))] = np.asarray(params[k], np.float32).reshape(-1)
        self.p.copy_(torch.from_numpy(flat))
        self.pack()

    def pack(self, stream=None) -> None:
        L = lib()
        for l in range(LAYERS):
            check(L.gpsat_gnn_pack(self.ptr(f"Wv3_{l}"), D, 3 * D, _p(self.fwd_v[l]), _p(self.bwd_v[l]), 3 * D,
                                   stream))
            check(L.gpsat_gnn_pack(self.ptr(f"Wc_{l}"), D, D, _p(self.fwd_c[l]), None, 0, stream))
            check(L.gpsat_gnn_pack(self.ptr(f"U_{l}"), D, 2 * D, _p(self.fwd_u[l]), _p(self.bwd_c[l]), 3 * D, stream))
            if l + 1 < LAYERS:
                check(L.gpsat_gnn_pack(self.ptr(f"Wc_{l + 1}"), D, D, None, _off(self.bwd_c[l], 2 * D), 3 * D, stream))
        check(L.gpsat_gnn_pack(self.ptr("Wc_0"), D, D, None, _p(self.bwd_c1), D, stream))
        check(L.gpsat_gnn_pack(self.ptr("Win"), D, D, _p(self.fwd_in), None, 0, stream))

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, stream=None) -> None:
        self.step += 1
        check(lib().gpsat_gnn_adam(_p(self.p), _p(self.g), _p(self.m), _p(self.v), self.n, lr, beta1, beta2, eps,
                                   self.step, stream))
        self.pack(stream)


# ---------------------------------------------------------------- forward / backward
class Pass:
    """Activations of one forward pass over a graph (kept for the backward)."""

    def __init__(self, net: SeedNet, g: Graph):
        import torch
        bf = dict(dtype=torch.bfloat16, device=g.device)
        V, C = max(g.V, 1), max(g.C, 1)
        self.net, self.g = net, g
        self.Hv = [torch.empty(V, D, **bf) for _ in range(LAYERS + 1)]
        self.Hc = [torch.empty(C, D, **bf) for _ in range(LAYERS + 1)]
        self.A3 = [torch.empty(V, 3 * D, **bf) for _ in range(LAYERS)]
        self.Zc = torch.empty(C, D, **bf)
        self.Bm = torch.empty(C, 2 * D, **bf)
        self.err = torch.zeros(1, dtype=torch.int32, device=g.device)

    def mm(self, X, ldx, rows, K, B, N, bias, Y, ldy, stream, relu=0):
        check(lib().gpsat_gnn_mm(X, ldx, rows, K, _p(B), B.stride(0), N, bias, relu, Y, ldy, _p(self.err),
                                 stream))

    def forward(self, stream=None):
        L, net, g = lib(), self.net, self.g
        V, C = g.V, g.C
        self.mm(_p(g.feat), D, V, D, net.fwd_in, D, net.ptr("bin"), _p(self.Hv[0]), D, stream, relu=1)
        check(L.gpsat_gnn_broadcast(net.ptr("hc0"), C, _p(self.Hc[0]), D, stream))
        for l in range(LAYERS):
            A3 = self.A3[l]
            self.mm(_p(self.Hv[l]), D, V, D, net.fwd_v[l], 3 * D, net.ptr(f"bias3_{l}"), _p(A3), 3 * D, stream)
            self.mm(_p(self.Hc[l]), D, C, D, net.fwd_c[l], D, net.ptr(f"bc_{l}"), _p(self.Zc), D, stream)
            check(L.gpsat_gnn_gather(_p(g.c_off), _p(g.c_edges), C, _p(A3), _off(A3, D), 3 * D, _p(g.c_scale),
                                     _p(self.Zc), D, _p(self.Hc[l + 1]), D, 1, stream))
            self.mm(_p(self.Hc[l + 1]), D, C, D, net.fwd_u[l], 2 * D, None, _p(self.Bm), 2 * D, stream)
            check(L.gpsat_gnn_gather(_p(g.v_off), _p(g.v_edges), V, _p(self.Bm), _off(self.Bm, D), 2 * D,
                                     _p(g.v_scale), _off(A3, 2 * D), 3 * D, _p(self.Hv[l + 1]), D, 1, stream))
        return self.Hv[LAYERS]

    def heads(self, score, phase, stream=None):
        check(lib().gpsat_gnn_head(_p(self.Hv[LAYERS]), D, self.g.V, self.net.ptr("head"), None, None, None, None,
                                   _p(score), _p(phase), None, 0, None, None, stream))

    def loss_backward(self, y_act, w_act, t_phase, w_phase, loss, stream=None):
        """Heads + losses, then the gradient of the summed loss into net.g."""
        import torch
        L, net, g = lib(), self.net, self.g
        V, C = g.V, g.C
        bf = dict(dtype=torch.bfloat16, device=g.device)
        dHv = torch.empty(max(V, 1), D, **bf)
        check(L.gpsat_gnn_head(_p(self.Hv[LAYERS]), D, V, net.ptr("head"), _p(y_act), _p(w_act), _p(t_phase),
                               _p(w_phase), None, None, _p(dHv), D, net.ptr("head", True), _p(loss), stream))
        GV = torch.empty(max(V, 1), 3 * D, **bf)                # [dA+ | dA- | dPreV]
        GC = [torch.empty(max(C, 1), 3 * D, **bf) for _ in range(2)]   # [dB+ | dB- | dPreC of the layer above]
        dHc = torch.empty(max(C, 1), D, **bf)
        for l in range(LAYERS - 1, -1, -1):
            gc, gc_next = GC[l % 2], GC[(l + 1) % 2]
            # through H_v^{l+1} = relu(sum B + Zv)
            check(L.gpsat_gnn_relu_bwd(_p(dHv), D, _p(self.Hv[l + 1]), D, V, _off(GV, 2 * D), 3 * D, stream))
            check(L.gpsat_gnn_gather_split(_p(g.c_off), _p(g.c_edges), C, _off(GV, 2 * D), 3 * D, _p(g.v_scale),
                                           _p(gc), _off(gc, D), 3 * D, stream))
            # H_c^{l+1} feeds B (this layer) and Zc of the layer above
            K = 3 * D if l + 1 < LAYERS else 2 * D
            self.mm(_p(gc), 3 * D, C, K, net.bwd_c[l], D, None, _p(dHc), D, stream)
            check(L.gpsat_gnn_wgrad(_p(self.Hc[l + 1]), D, _p(gc), 3 * D, C, 2 * D, net.ptr(f"U_{l}", True),
                                    _p(self.err), stream))
            # through H_c^{l+1} = relu(sum A + Zc); dPreC goes to the other buffer's last third
            check(L.gpsat_gnn_relu_bwd(_p(dHc), D, _p(self.Hc[l + 1]), D, C, _off(gc_next, 2 * D), 3 * D, stream))
            check(L.gpsat_gnn_wgrad(_p(self.Hc[l]), D, _off(gc_next, 2 * D), 3 * D, C, D, net.ptr(f"Wc_{l}", True),
                                    _p(self.err), stream))
            check(L.gpsat_gnn_colsum(_off(gc_next, 2 * D), 3 * D, C, net.ptr(f"bc_{l}", True), stream))
            check(L.gpsat_gnn_gather_split(_p(g.v_off), _p(g.v_edges), V, _off(gc_next, 2 * D), 3 * D,
                                           _p(g.c_scale), _p(GV), _off(GV, D), 3 * D, stream))
            # A3 = H_v^l Wv3 + bias3
            check(L.gpsat_gnn_wgrad(_p(self.Hv[l]), D, _p(GV), 3 * D, V, 3 * D, net.ptr(f"Wv3_{l}", True),
                                    _p(self.err), stream))
            check(L.gpsat_gnn_colsum(_off(GV, 2 * D), 3 * D, V, net.ptr(f"bias3_{l}", True) + 4 * 2 * D, stream))
            self.mm(_p(GV), 3 * D, V, 3 * D, net.bwd_v[l], D, None, _p(dHv), D, stream)
            if l == 0:
                # H_c^0 = hc0 feeds only Zc of layer 0
                self.mm(_off(gc_next, 2 * D), 3 * D, C, D, net.bwd_c1, D, None, _p(dHc), D, stream)
                check(L.gpsat_gnn_colsum(_p(dHc), D, C, net.ptr("hc0", True), stream))
                # H_v^0 = relu(F Win + bin)
                check(L.gpsat_gnn_relu_bwd(_p(dHv), D, _p(self.Hv[0]), D, V, _p(dHv), D, stream))
                check(L.gpsat_gnn_wgrad(_p(g.feat), D, _p(dHv), D, V, D, net.ptr("Win", True), _p(self.err), stream))
                check(L.gpsat_gnn_colsum(_p(dHv), D, V, net.ptr("bin", True), stream))


# ---------------------------------------------------------------- labels and seeds
def participation_targets(formulas, n_vars, conflict_budget=20000, options=None):
    """Solves every formula once, logging per-variable conflict participation
    and learnt-clause occurrences.  Returns per-variable arrays (all formulas
    concatenated): activity target y = mean of log1p(count) / log1p(max count
    of its formula) over the two counts, phase target (1 where the model sets
    the variable true; SAT formulas only), and the solve output."""
    from . import Batch, solve_options
    b = Batch(formulas, n_vars)
    o = options or solve_options(conflict_budget=conflict_budget)
    out = b.solve(o, participation=2)
    counts = (out["participation"].astype(np.float64), out["learnt_occurrences"].astype(np.float64))
    part = counts[0]
    y = np.zeros(len(part), np.float32)
    t = np.zeros(len(part), np.float32)
    has_phase = np.zeros(len(part), bool)
    for f in range(b.n_formulas):
        a, e = b.var_off[f], b.var_off[f + 1]
        for c in counts:
            mx = c[a:e].max() if e > a else 0
            if mx > 0:
                y[a:e] += 0.5 * (np.log1p(c[a:e]) / np.log1p(mx)).astype(np.float32)
        if out["verdict"][f] == 10:
            t[a:e] = (out["model"][a:e] > 0)
            has_phase[a:e] = True
    return y, t, has_phase, out


def seeds_from(score: np.ndarray, phase: np.ndarray, scale: float = 5.0):
    """VSIDS activity seeds (scale * sigmoid(score)) and saved phases (1 = true)."""
    act = (scale / (1.0 + np.exp(-score.astype(np.float64)))).astype(np.float32)
    return act, (phase > 0).astype(np.int8)


def predict(net: SeedNet, formulas, n_vars, stream=None, communities=None):
    """Per-variable (score, phase logit) for every formula, concatenated."""
    import torch
    g = Graph(formulas, n_vars, net.device, communities)
    ps = Pass(net, g)
    ps.forward(stream)
    score = torch.empty(max(g.V, 1), dtype=torch.float32, device=net.device)
    phase = torch.empty(max(g.V, 1), dtype=torch.float32, device=net.device)
    ps.heads(score, phase, stream)
    torch.cuda.synchronize()
    if int(ps.err.item()):
        raise RuntimeError("gnn: a matrix-product tile gave up waiting")
    return score[:g.V].cpu().numpy(), phase[:g.V].cpu().numpy()


def train_step(net: SeedNet, formulas, n_vars, y, t, has_phase, lr=1e-3, stream=None, communities=None):
    """One Adam step on a batch of formulas; returns (activity loss, phase loss)."""
    import torch
    g = Graph(formulas, n_vars, net.device, communities)
    dev = net.device
    nf = len(formulas)
    counts = np.repeat(np.asarray(n_vars, np.float64), np.asarray(n_vars, np.int64))
    w_act = (1.0 / (counts * nf)).astype(np.float32)
    n_sat = max(1, len({f for f in range(nf) if has_phase[g.var_base[f]:g.var_base[f + 1]].any()}))
    w_ph = np.where(has_phase, 1.0 / (counts * n_sat), 0.0).astype(np.float32)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)
    ps = Pass(net, g)
    ps.forward(stream)
    loss = torch.zeros(2, dtype=torch.float32, device=dev)
    ps.loss_backward(T(y), T(w_act), T(t), T(w_ph), loss, stream)
    net.adam(lr=lr, stream=stream)
    torch.cuda.synchronize()
    if int(ps.err.item()):
        raise RuntimeError("gnn: a matrix-product tile gave up waiting")
    l = loss.cpu().numpy()
    return float(l[0]), float(l[1])


# ---------------------------------------------------------------- workloads
def communities_of(n: int, groups: int = 40) -> np.ndarray:
    """Community id of each variable of a planted instance (equal contiguous blocks)."""
    return (np.arange(n, dtype=np.int64) * groups // n).astype(np.float32)


def training_set(count: int, seed: int = 0, kind: str = "random"):
    """Training formulas as (n, lits, offsets, communities or None).

    "random":  random k-SAT near the satisfiability thresholds, k in {3, 4, 5}
               with clause ratios 4.26 / 9.93 / 21.1, n ~ U[100, 400]; formula i
               uses generator seed 20000 + seed * 1000003 + i.
    "planted": planted community 3-SAT as the structured workload generates it
               (ratio 4.0, 40 communities, 90% of a clause in one), smaller:
               n ~ U[500, 3000]; formula i uses seed 60000 + seed * 1000003 + i.
    """
    from . import gen_planted, gen_random_ksat
    rng = np.random.default_rng(seed)
    out = []
    if kind == "random":
        ks = rng.choice([3, 4, 5], size=count)
        ns = rng.integers(100, 401, size=count)
        ratio = {3: 4.26, 4: 9.93, 5: 21.1}
        for i, (k, n) in enumerate(zip(ks, ns)):
            lits, off = gen_random_ksat(20000 + seed * 1000003 + i, int(n), int(round(ratio[int(k)] * n)), int(k))
            out.append((int(n), lits, off, None))
    elif kind == "planted":
        ns = rng.integers(500, 3001, size=count)
        for i, n in enumerate(ns):
            lits, off, _ = gen_planted(60000 + seed * 1000003 + i, int(n), 4 * int(n), 3, 40, 0.9)
            out.append((int(n), lits, off, communities_of(int(n))))
    else:
        raise ValueError(f"unknown training set {kind!r}")
    return out


def train(net: SeedNet, data, epochs: int = 3, batch: int = 256, lr: float = 2e-3, conflict_budget: int = 20000,
          log=print):
    """Labels every formula with the solver, then trains for `epochs` passes.
    data: (n, lits, offsets[, communities]) tuples."""
    formulas = [(d[1], d[2]) for d in data]
    nv = [d[0] for d in data]
    comm = [d[3] if len(d) > 3 else None for d in data]
    use_comm = any(c is not None for c in comm)
    y, t, has_phase, out = participation_targets(formulas, nv, conflict_budget)
    base = np.zeros(len(nv) + 1, np.int64)
    base[1:] = np.cumsum(nv)
    rng = np.random.default_rng(1)
    hist = []
    for ep in range(epochs):
        order = rng.permutation(len(formulas))
        tot = np.zeros(2)
        for b0 in range(0, len(order), batch):
            idx = order[b0:b0 + batch]
            sel = np.concatenate([np.arange(base[i], base[i + 1]) for i in idx])
            cm = [comm[i] if comm[i] is not None else np.zeros(nv[i], np.float32) for i in idx] if use_comm else None
            la, lp = train_step(net, [formulas[i] for i in idx], [nv[i] for i in idx], y[sel], t[sel],
                                has_phase[sel], lr=lr, communities=cm)
            tot += (la, lp)
        nb = (len(order) + batch - 1) // batch
        hist.append(tot / nb)
        if log:
            log(f"epoch {ep}: activity loss {tot[0] / nb:.4f}  phase loss {tot[1] / nb:.4f}")
    return hist, out
