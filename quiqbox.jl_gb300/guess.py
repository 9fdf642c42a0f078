"""Learned initial guess for closed-shell SCF (minimal basis, H/C/N/O).

A small MLP predicts the converged per-spin density block of every atom pair (and of
every atom with itself) from pair features; the blocks assemble into an initial
density for runHartreeFockBatched, which then converges it like any other guess (the
final energy is always the SCF's own).  There is no counterpart in the reference,
whose guesses are CoreH / GWH / SAD / Direct (src/HartreeFock.jl:162-293); the seam it
plugs into is the initial-density input of the batched SCF, the analogue of
OrbCoeffInitialConfig(:Direct) (HartreeFock.jl:162-172).

Network: 128 inputs -> 4 hidden layers of width 256 with GELU -> 64 outputs (25 used: a
5 x 5 block), BF16 weights and activations, FP32 accumulation and FP32 master weights
for Adam.  Every GPU operation is a kernel of this library (csrc/mlp.cu) called through
the C ABI; torch only provides device memory and the stream.

Features of the pair (A, B) are described at pair_data; blocks live in a local frame
(z along A -> B, x towards a neighbouring atom), so the p components are predicted
frame-independently and rotated back (D_lab = T_A D_loc T_B^T with T = diag(1, 1, R)).
"""
from __future__ import annotations

import ctypes as C
import json
import math
import time
from pathlib import Path

import numpy as np

ELEMENTS = ("H", "C", "N", "O")
NBASIS = {"H": 1, "C": 5, "N": 5, "O": 5}
NIN, NHID, NLAYER, NOUT = 128, 256, 4, 64
NFEAT = 74
MU = 0.25 + 0.25 * np.arange(32)
WEIGHTS_FILE = Path(__file__).resolve().parent / "data" / "guess_mlp.npz"


# ---------------------------------------------------------------------------
# features and blocks, vectorised over every atom pair of every molecule
def pair_list(symbols):
    return [(a, b) for a in range(len(symbols)) for b in range(a, len(symbols))]


def atom_offsets(symbols):
    off, o = [], 0
    for s in symbols:
        off.append(o)
        o += NBASIS[s]
    return off, o


def _unit(v):
    return v / np.maximum(np.linalg.norm(v, axis=-1, keepdims=True), 1e-300)


def pair_data(mols):
    """Pairs (a <= b) of every molecule with their local frames and features.

    Local frame: for a != b, z along A -> B and x towards the atom nearest the bond
    midpoint (its component perpendicular to z); for a == b, z towards the nearest
    neighbour and x towards the second nearest.  Without such an atom x is any unit
    vector perpendicular to z.  Features (74 used of NIN): 32 Gaussian-expanded r_AB, a
    same-atom flag, element one-hots of A and B, per endpoint and per element of the
    neighbours sum w (1, cos_z, cos_x, (3 cos_z^2 - 1) / 2) with w = exp(-(r / 2.5)^2)
    in the local frame, and the molecular charge."""
    nats = np.array([len(m["symbols"]) for m in mols])
    nat = int(nats.max())
    nm = len(mols)
    pos = np.zeros((nm, nat, 3))
    el = np.full((nm, nat), -1, np.int64)
    code = {e: i for i, e in enumerate(ELEMENTS)}
    for k, m in enumerate(mols):
        na = nats[k]
        pos[k, :na] = m["coords"]
        el[k, :na] = [code[x] for x in m["symbols"]]
    tri = {n: np.triu_indices(n) for n in np.unique(nats)}
    cnt = nats * (nats + 1) // 2
    pm = np.repeat(np.arange(nm), cnt)
    pa = np.concatenate([tri[n][0] for n in nats])
    pb = np.concatenate([tri[n][1] for n in nats])
    npair = len(pm)
    PA, PB = pos[pm, pa], pos[pm, pb]
    same = pa == pb
    neigh = pos[pm]                                   # (npair, nat, 3)
    nel = el[pm]                                      # (npair, nat)
    valid = nel >= 0
    idx = np.arange(nat)[None, :]
    dA = np.linalg.norm(neigh - PA[:, None, :], axis=2)
    # z axis
    z = _unit(PB - PA)
    dA_other = np.where(valid & (idx != pa[:, None]), dA, np.inf)
    order = np.argsort(dA_other, axis=1)
    n1 = order[:, 0]
    z_same = _unit(neigh[np.arange(npair), n1] - PA)
    has1 = np.isfinite(dA_other[np.arange(npair), n1])
    z = np.where(same[:, None], np.where(has1[:, None], z_same, np.array([0.0, 0.0, 1.0])), z)
    # x axis: reference atom (midpoint-nearest third atom, or second-nearest neighbour)
    mid = 0.5 * (PA + PB)
    dmid = np.linalg.norm(neigh - mid[:, None, :], axis=2)
    excl = (idx == pa[:, None]) | (idx == pb[:, None])
    rel = neigh - PA[:, None, :]
    perp = rel - np.sum(rel * z[:, None, :], axis=2, keepdims=True) * z[:, None, :]
    pn = np.linalg.norm(perp, axis=2)
    cand_pair = np.where(valid & ~excl & (pn > 0.3), dmid, np.inf)
    cand_same = np.where(valid & (idx != pa[:, None]) & (idx != n1[:, None]) & (pn > 0.3), dA, np.inf)
    cand = np.where(same[:, None], cand_same, cand_pair)
    ref_i = np.argmin(cand, axis=1)
    has_ref = np.isfinite(cand[np.arange(npair), ref_i])
    xr = perp[np.arange(npair), ref_i]
    helper = np.where(np.abs(z[:, 2:3]) < 0.9, np.array([0.0, 0.0, 1.0]), np.array([1.0, 0.0, 0.0]))
    xa = np.cross(helper, z)
    x = _unit(np.where(has_ref[:, None], xr, xa))
    y = np.cross(z, x)
    R = np.stack([x, y, z], axis=2)                  # columns: local axes in lab coordinates
    # features
    X = np.zeros((npair, NIN), np.float32)
    r = np.linalg.norm(PB - PA, axis=1)
    X[:, :32] = np.exp(-((r[:, None] - MU[None, :]) / 0.25) ** 2)
    X[:, 32] = same
    X[np.arange(npair), 33 + el[pm, pa]] = 1.0
    X[np.arange(npair), 37 + el[pm, pb]] = 1.0
    for e_off, (P, me) in enumerate(((PA, pa), (PB, pb))):
        u = neigh - P[:, None, :]
        d = np.linalg.norm(u, axis=2)
        w = np.where(valid & (idx != me[:, None]), np.exp(-(d / 2.5) ** 2), 0.0)
        dn = np.maximum(d, 1e-12)
        cz = np.sum(u * z[:, None, :], axis=2) / dn
        cx = np.sum(u * x[:, None, :], axis=2) / dn
        terms = np.stack([w, w * cz, w * cx, w * 0.5 * (3 * cz * cz - 1)], axis=2)   # (npair, nat, 4)
        for e in range(4):
            sel = (nel == e)[:, :, None]
            X[:, 41 + 16 * e_off + 4 * e:41 + 16 * e_off + 4 * e + 4] = np.sum(terms * sel, axis=1)
    X[:, 73] = np.array([m["charge"] for m in mols], np.float32)[pm]
    return {"mol": pm, "a": pa, "b": pb, "R": R, "X": X}


def _gather_index(symbols):
    """Per atom the 5 function indices of its padded block (n = dummy row/column)."""
    off, n = atom_offsets(symbols)
    out = np.full((len(symbols), 5), n, np.int64)
    for i, sy in enumerate(symbols):
        out[i, :NBASIS[sy]] = off[i] + np.arange(NBASIS[sy])
    return out, n


def _T5(R):
    T = np.zeros((R.shape[0], 5, 5))
    T[:, 0, 0] = T[:, 1, 1] = 1.0
    T[:, 2:, 2:] = R
    return T


def blocks_from_densities(mols, dens, pd):
    """Local-frame blocks (targets) and their masks, (npair, 64) each."""
    Y = np.zeros((len(pd["mol"]), NOUT), np.float32)
    Wm = np.zeros_like(Y)
    T = _T5(pd["R"])
    start = 0
    for k, (m, D) in enumerate(zip(mols, dens)):
        gi, n = _gather_index(m["symbols"])
        cnt = len(m["symbols"]) * (len(m["symbols"]) + 1) // 2
        sl = slice(start, start + cnt)
        Dp = np.zeros((n + 1, n + 1))
        Dp[:n, :n] = D
        ia, ib = gi[pd["a"][sl]], gi[pd["b"][sl]]
        blk = Dp[ia[:, :, None], ib[:, None, :]]
        loc = np.einsum("pji,pjk,pkl->pil", T[sl], blk, T[sl])
        mask = ((ia < n)[:, :, None] & (ib < n)[:, None, :]).astype(np.float32)
        Y[sl, :25] = (loc * mask).reshape(cnt, 25)
        Wm[sl, :25] = mask.reshape(cnt, 25)
        start += cnt
    return Y, Wm


def densities_from_blocks(mols, pd, Ypred):
    T = _T5(pd["R"])
    out, start = [], 0
    for m in mols:
        gi, n = _gather_index(m["symbols"])
        cnt = len(m["symbols"]) * (len(m["symbols"]) + 1) // 2
        sl = slice(start, start + cnt)
        loc = np.asarray(Ypred[sl, :25], float).reshape(cnt, 5, 5)
        blk = np.einsum("pij,pjk,plk->pil", T[sl], loc, T[sl])
        a, b = pd["a"][sl], pd["b"][sl]
        diag = a == b
        blk[diag] = 0.5 * (blk[diag] + np.transpose(blk[diag], (0, 2, 1)))
        Dp = np.zeros((n + 1, n + 1))
        ia, ib = gi[a], gi[b]
        Dp[ib[:, :, None], ia[:, None, :]] = np.transpose(blk, (0, 2, 1))
        Dp[ia[:, :, None], ib[:, None, :]] = blk
        out.append(Dp[:n, :n].copy())
        start += cnt
    return out


# ---------------------------------------------------------------------------
# the network on the GPU
def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _fp(t):
    return C.cast(t.data_ptr(), C.POINTER(C.c_float))


class GuessMLP:
    """Weights as FP32 masters + BF16 copies on the GPU; forward / backward / Adam through
    the library's kernels."""

    def __init__(self, lib, device="cuda:0", seed=0, params=None):
        import torch
        self.torch = torch
        self.lib = lib
        self.dev = torch.device(device)
        dims = [NIN] + [NHID] * NLAYER + [NOUT]
        self.dims = dims
        rng = np.random.default_rng(seed)
        self.W, self.b, self.Wb = [], [], []
        for l in range(len(dims) - 1):
            fan_in = dims[l]
            if params is None:
                w = rng.normal(0.0, math.sqrt(2.0 / fan_in), (dims[l + 1], dims[l])).astype(np.float32)
                bb = np.zeros(dims[l + 1], np.float32)
            else:
                w, bb = params["W%d" % l].astype(np.float32), params["b%d" % l].astype(np.float32)
            self.W.append(torch.tensor(w, device=self.dev))
            self.b.append(torch.tensor(bb, device=self.dev))
            self.Wb.append(torch.empty(w.shape, dtype=torch.bfloat16, device=self.dev))
        self.m = [torch.zeros_like(w) for w in self.W] + [torch.zeros_like(b) for b in self.b]
        self.v = [torch.zeros_like(w) for w in self.W] + [torch.zeros_like(b) for b in self.b]
        self.step_count = 0
        self.stream = C.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        self.refresh_bf16()

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"MLP kernel failed with status {rc}")

    def refresh_bf16(self):
        for w, wb in zip(self.W, self.Wb):
            self._check(self.lib.qb_f32_to_bf16(w.shape[0], w.shape[1], _fp(w), _ptr(wb), 0, self.stream))

    def gemm(self, A, B, bias, M, N, K):
        out = self.torch.empty((M, N), dtype=self.torch.float32, device=self.dev)
        self._check(self.lib.qb_bf16_gemm_nt(M, N, K, _ptr(A), _ptr(B), _fp(bias) if bias is not None else None,
                                             _fp(out), self.stream))
        return out

    def to_bf16(self, x, transpose=False):
        r, c = x.shape
        y = self.torch.empty((c, r) if transpose else (r, c), dtype=self.torch.bfloat16, device=self.dev)
        self._check(self.lib.qb_f32_to_bf16(r, c, _fp(x), _ptr(y), 1 if transpose else 0, self.stream))
        return y

    def transpose_bf16(self, x):
        r, c = x.shape
        y = self.torch.empty((c, r), dtype=self.torch.bfloat16, device=self.dev)
        self._check(self.lib.qb_bf16_transpose(r, c, _ptr(x), _ptr(y), self.stream))
        return y

    def forward(self, Xb):
        """Xb: (M, 64) bf16 on the device, M a multiple of 64.  Returns Y (fp32) and the
        saved activations."""
        M = Xb.shape[0]
        acts, zs = [Xb], []
        x = Xb
        L = len(self.W)
        for l in range(L):
            z = self.gemm(x, self.Wb[l], self.b[l], M, self.dims[l + 1], self.dims[l])
            if l == L - 1:
                return z, (acts, zs)
            a = self.torch.empty(z.shape, dtype=self.torch.bfloat16, device=self.dev)
            self._check(self.lib.qb_gelu_forward(z.numel(), _fp(z), _ptr(a), self.stream))
            zs.append(z)
            acts.append(a)
            x = a

    def backward(self, dY, saved):
        """Gradients (dW list, db list) of the loss whose gradient w.r.t. Y is dY (fp32)."""
        acts, zs = saved
        M = dY.shape[0]
        L = len(self.W)
        dWs, dbs = [None] * L, [None] * L
        d = dY
        for l in range(L - 1, -1, -1):
            db = self.torch.empty(self.dims[l + 1], dtype=self.torch.float32, device=self.dev)
            self._check(self.lib.qb_colsum(M, self.dims[l + 1], _fp(d), _fp(db), self.stream))
            dT = self.to_bf16(d, transpose=True)                 # (N_out, M)
            xT = self.transpose_bf16(acts[l])                    # (N_in, M)
            dWs[l] = self.gemm(dT, xT, None, self.dims[l + 1], self.dims[l], M)   # dZ^T X
            dbs[l] = db
            if l == 0:
                break
            db16 = self.to_bf16(d)                               # (M, N_out)
            wT = self.transpose_bf16(self.Wb[l])                 # (N_in, N_out)
            dx = self.gemm(db16, wT, None, M, self.dims[l], self.dims[l + 1])     # dZ W
            dz = self.torch.empty_like(dx)
            self._check(self.lib.qb_gelu_backward(dx.numel(), _fp(zs[l - 1]), _fp(dx), _fp(dz), self.stream))
            d = dz
        return dWs, dbs

    def loss_grad(self, Y, T, Wt):
        dY = self.torch.empty_like(Y)
        loss = self.torch.zeros(1, dtype=self.torch.float32, device=self.dev)
        wsum = float(Wt.sum().item())
        self._check(self.lib.qb_mse_grad(Y.numel(), _fp(Y), _fp(T), _fp(Wt), C.c_float(wsum), _fp(dY), _fp(loss),
                                         self.stream))
        return loss, dY

    def adam(self, dWs, dbs, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        L = len(self.W)
        for l in range(L):
            self._check(self.lib.qb_adam_step(self.W[l].numel(), _fp(self.W[l]), _fp(dWs[l]), _fp(self.m[l]),
                                              _fp(self.v[l]), _ptr(self.Wb[l]), C.c_float(lr), C.c_float(b1),
                                              C.c_float(b2), C.c_float(eps), self.step_count, self.stream))
            self._check(self.lib.qb_adam_step(self.b[l].numel(), _fp(self.b[l]), _fp(dbs[l]), _fp(self.m[L + l]),
                                              _fp(self.v[L + l]), None, C.c_float(lr), C.c_float(b1), C.c_float(b2),
                                              C.c_float(eps), self.step_count, self.stream))

    def params(self):
        out = {}
        for l in range(len(self.W)):
            out["W%d" % l] = self.W[l].cpu().numpy()
            out["b%d" % l] = self.b[l].cpu().numpy()
        return out

    def predict(self, X):
        """X (n, 64) float32 numpy -> (n, 64) float32 numpy."""
        torch = self.torch
        n = X.shape[0]
        M = max(64, ((n + 63) // 64) * 64)
        Xp = np.zeros((M, NIN), np.float32)
        Xp[:n] = X
        x = torch.tensor(Xp, device=self.dev)
        Y, _ = self.forward(self.to_bf16(x))
        return Y[:n].cpu().numpy()


def _pad_rows(a, mult=64):
    n = a.shape[0]
    M = ((n + mult - 1) // mult) * mult
    if M == n:
        return a
    out = np.zeros((M,) + a.shape[1:], a.dtype)
    out[:n] = a
    return out


# ---------------------------------------------------------------------------
def dataset(mols, densities):
    pd = pair_data(mols)
    Y, W = blocks_from_densities(mols, densities, pd)
    return pd["X"], Y, W


def train(net, X, Y, W, epochs=20, batch=4096, lr=1e-3, seed=0, log=None):
    torch = net.torch
    rng = np.random.default_rng(seed)
    n = X.shape[0]
    Xd = torch.tensor(X, device=net.dev)
    Yd = torch.tensor(Y, device=net.dev)
    Wd = torch.tensor(W, device=net.dev)
    history = []
    for ep in range(epochs):
        perm = torch.tensor(rng.permutation(n), device=net.dev)
        tot = 0.0
        nb = 0
        lr_ep = lr * (0.5 * (1 + math.cos(math.pi * ep / epochs)))
        for s in range(0, n - batch + 1, batch):
            idx = perm[s:s + batch]
            xb = net.to_bf16(Xd[idx].contiguous())
            Yp, saved = net.forward(xb)
            loss, dY = net.loss_grad(Yp, Yd[idx].contiguous(), Wd[idx].contiguous())
            dWs, dbs = net.backward(dY, saved)
            net.adam(dWs, dbs, lr=lr_ep)
            tot += float(loss.item())
            nb += 1
        history.append(tot / max(nb, 1))
        if log:
            log(f"epoch {ep} loss {history[-1]:.3e}")
    return history


def load(lib, device="cuda:0", path=WEIGHTS_FILE):
    p = np.load(path)
    return GuessMLP(lib, device, params={k: p[k] for k in p.files if k[0] in "Wb"})


def initial_densities(net, mols):
    """Learned initial per-spin densities of a list of generated molecules."""
    pd = pair_data(mols)
    return densities_from_blocks(mols, pd, net.predict(pd["X"]))


def train_main(n_train=20000, n_test=2000, seed_train=101, seed_test=202, epochs=20, out=WEIGHTS_FILE,
               report=None):
    """Labels from the plain batched GPU SCF, training with the library's kernels, held-out
    evaluation (iterations and wall time, CoreH vs learned), weights saved to `out`."""
    import __graft_entry__ as ge
    qb = ge.load_package()
    from quiqbox_gb300 import _lib as L
    from quiqbox_gb300.workloads import batch_molecules
    lib = L.load()
    t0 = time.time()
    mols = batch_molecules(n_train, seed=seed_train, atoms=(3, 12), basis_names=("STO-3G",))
    dens, keep = [], []
    for s in range(0, n_train, 512):
        chunk = mols[s:s + 512]
        res = qb.runHartreeFockBatched([(m["nuc"], m["flat"], m["charge"]) for m in chunk], return_densities=True)
        for k, m in enumerate(chunk):
            if res.converged[k]:
                keep.append(m)
                dens.append(res.densities[k])
    t_label = time.time() - t0
    X, Y, W = dataset(keep, dens)
    net = GuessMLP(lib, seed=0)
    t1 = time.time()
    hist = train(net, X, Y, W, epochs=epochs, log=print)
    t_train = time.time() - t1
    params = net.params()
    out = Path(out)
    out.parent.mkdir(parents=True, exist_ok=True)
    np.savez(out, **params, meta=json.dumps({"n_train_molecules": len(keep), "pairs": int(X.shape[0]),
                                             "epochs": epochs, "final_loss": hist[-1]}))
    ev = evaluate(qb, net, n_test, seed_test)
    info = {"label_s": t_label, "train_s": t_train, "train_molecules": len(keep), "train_pairs": int(X.shape[0]),
            "loss_first": hist[0], "loss_last": hist[-1], "eval": ev}
    if report:
        Path(report).write_text(json.dumps(info, indent=1))
    return info


def solve_with_guess(qb, net, mols, fallback=True, first_max_iter=100):
    """Batched SCF from the learned guess; molecules it has not converged after
    `first_max_iter` iterations are solved again from the core-Hamiltonian guess (the
    fallback).  Returns (result, fallback indices)."""
    args = [(m["nuc"], m["flat"], m["charge"]) for m in mols]
    D0 = initial_densities(net, mols)
    cfg = qb.BatchSCFConfig(max_iter=first_max_iter if fallback else 200)
    res = qb.runHartreeFockBatched(args, config=cfg, initial_densities=D0)
    redo = [k for k in range(len(mols)) if not res.converged[k]] if fallback else []
    if redo:
        r2 = qb.runHartreeFockBatched([args[k] for k in redo])
        for j, k in enumerate(redo):
            res.energies[k] = r2.energies[j]
            res.elec_energies[k] = r2.elec_energies[j]
            res.iterations[k] += r2.iterations[j]
            res.converged[k] = r2.converged[j]
    return res, redo


def evaluate(qb, net, n_test=2000, seed=202):
    from quiqbox_gb300.workloads import batch_molecules
    mols = batch_molecules(n_test, seed=seed, atoms=(3, 12), basis_names=("STO-3G",))
    args = [(m["nuc"], m["flat"], m["charge"]) for m in mols]
    qb.runHartreeFockBatched(args[:16])   # warm-up
    t0 = time.perf_counter()
    base = qb.runHartreeFockBatched(args)
    t_base = time.perf_counter() - t0
    t0 = time.perf_counter()
    lrn, redo = solve_with_guess(qb, net, mols)
    t_lrn = time.perf_counter() - t0
    both = base.converged & lrn.converged
    dE = np.abs(base.energies[both] - lrn.energies[both])
    return {"molecules": n_test, "coreh_converged": int(base.converged.sum()),
            "learned_converged": int(lrn.converged.sum()), "fallback": len(redo),
            "coreh_mean_iterations": float(base.iterations[both].mean()),
            "learned_mean_iterations": float(lrn.iterations[both].mean()),
            "coreh_wall_s": t_base, "learned_wall_s": t_lrn,
            "coreh_solves_per_s": float(base.converged.sum() / t_base),
            "learned_solves_per_s": float(lrn.converged.sum() / t_lrn),
            "max_abs_dE_same_state": float(np.sort(dE)[int(0.99 * len(dE))]) if len(dE) else None,
            "frac_same_state_1e-8": float((dE < 1e-8).mean()) if len(dE) else None}
