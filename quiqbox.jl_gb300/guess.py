"""Learned initial guess for closed-shell SCF (minimal basis, H/C/N/O).

A small MLP predicts the converged per-spin density block of every atom pair (and of
every atom with itself) from pair features; the blocks assemble into an initial
density for runHartreeFockBatched, which then converges it like any other guess (the
final energy is always the SCF's own).  There is no counterpart in the reference,
whose guesses are CoreH / GWH / SAD / Direct (src/HartreeFock.jl:162-293); the seam it
plugs into is the initial-density input of the batched SCF, the analogue of
OrbCoeffInitialConfig(:Direct) (HartreeFock.jl:162-172).

Network: 64 inputs -> 4 hidden layers of width 256 with GELU -> 64 outputs (25 used: a
5 x 5 block), BF16 weights and activations, FP32 accumulation and FP32 master weights
for Adam.  Every GPU operation is a kernel of this library (csrc/mlp.cu) called through
the C ABI; torch only provides device memory and the stream.

Features of the pair (A, B) (49 used, padded to 64): 32 Gaussian-expanded distances
exp(-((r_AB - mu_k) / 0.25)^2), mu_k = 0.25 .. 8 bohr; a same-atom flag; element
one-hots of A and B; per endpoint a smooth count of neighbouring H/C/N/O atoms
(sum exp(-(r / 2.5)^2)).  Blocks live in a local frame whose z axis is A -> B, so the
p components are predicted frame-independently and rotated back (D_lab = T_A D_loc T_B^T
with T = diag(1, 1, R)).
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
NIN, NHID, NLAYER, NOUT = 64, 256, 4, 64
NFEAT = 49
MU = 0.25 + 0.25 * np.arange(32)
WEIGHTS_FILE = Path(__file__).resolve().parent / "data" / "guess_mlp.npz"


# ---------------------------------------------------------------------------
# features and blocks
def _frame(ra, rb):
    """Rotation R (columns = local x, y, z axes in lab coordinates); z along A -> B."""
    d = np.asarray(rb, float) - np.asarray(ra, float)
    r = np.linalg.norm(d)
    if r < 1e-12:
        return np.eye(3)
    z = d / r
    ref = np.array([0.0, 0.0, 1.0]) if abs(z[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    x = np.cross(ref, z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    return np.stack([x, y, z], axis=1)


def _T(sym, R):
    n = NBASIS[sym]
    T = np.eye(n)
    if n == 5:
        T[2:, 2:] = R
    return T


def atom_offsets(symbols):
    off, o = [], 0
    for s in symbols:
        off.append(o)
        o += NBASIS[s]
    return off, o


def pair_list(symbols):
    return [(a, b) for a in range(len(symbols)) for b in range(a, len(symbols))]


def features(symbols, coords):
    """(npairs, 64) float32 features of pair_list(symbols)."""
    P = np.asarray(coords, float)
    nat = len(symbols)
    oh = np.zeros((nat, 4))
    for i, s in enumerate(symbols):
        oh[i, ELEMENTS.index(s)] = 1.0
    dist = np.linalg.norm(P[:, None, :] - P[None, :, :], axis=2)
    env = np.zeros((nat, 4))
    for i in range(nat):
        w = np.exp(-(dist[i] / 2.5) ** 2)
        w[i] = 0.0
        env[i] = w @ oh
    pairs = pair_list(symbols)
    X = np.zeros((len(pairs), NIN), np.float32)
    for k, (a, b) in enumerate(pairs):
        r = dist[a, b]
        X[k, :32] = np.exp(-((r - MU) / 0.25) ** 2)
        X[k, 32] = 1.0 if a == b else 0.0
        X[k, 33:37] = oh[a]
        X[k, 37:41] = oh[b]
        X[k, 41:45] = env[a]
        X[k, 45:49] = env[b]
    return X


def blocks_from_density(symbols, coords, D):
    """Targets (npairs, 64) and weights (npairs, 64): local-frame blocks of D."""
    off, _ = atom_offsets(symbols)
    pairs = pair_list(symbols)
    Y = np.zeros((len(pairs), NOUT), np.float32)
    W = np.zeros((len(pairs), NOUT), np.float32)
    for k, (a, b) in enumerate(pairs):
        R = _frame(coords[a], coords[b])
        na, nb = NBASIS[symbols[a]], NBASIS[symbols[b]]
        blk = D[off[a]:off[a] + na, off[b]:off[b] + nb]
        loc = _T(symbols[a], R).T @ blk @ _T(symbols[b], R)
        full = np.zeros((5, 5))
        full[:na, :nb] = loc
        msk = np.zeros((5, 5))
        msk[:na, :nb] = 1.0
        Y[k, :25] = full.reshape(-1)
        W[k, :25] = msk.reshape(-1)
    return Y, W


def density_from_blocks(symbols, coords, Ypred):
    """Symmetric density assembled from predicted local-frame blocks."""
    off, n = atom_offsets(symbols)
    D = np.zeros((n, n))
    for k, (a, b) in enumerate(pair_list(symbols)):
        R = _frame(coords[a], coords[b])
        na, nb = NBASIS[symbols[a]], NBASIS[symbols[b]]
        loc = np.asarray(Ypred[k, :25], float).reshape(5, 5)[:na, :nb]
        blk = _T(symbols[a], R) @ loc @ _T(symbols[b], R).T
        if a == b:
            blk = 0.5 * (blk + blk.T)
        D[off[a]:off[a] + na, off[b]:off[b] + nb] = blk
        D[off[b]:off[b] + nb, off[a]:off[a] + na] = blk.T
    return D


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
    X, Y, W = [], [], []
    for m, D in zip(mols, densities):
        X.append(features(m["symbols"], m["coords"]))
        y, w = blocks_from_density(m["symbols"], m["coords"], D)
        Y.append(y)
        W.append(w)
    return np.concatenate(X), np.concatenate(Y), np.concatenate(W)


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
    X = [features(m["symbols"], m["coords"]) for m in mols]
    counts = [x.shape[0] for x in X]
    Yp = net.predict(np.concatenate(X))
    out, o = [], 0
    for m, c in zip(mols, counts):
        out.append(density_from_blocks(m["symbols"], m["coords"], Yp[o:o + c]))
        o += c
    return out


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


def solve_with_guess(qb, net, mols, fallback=True):
    """Batched SCF from the learned guess; molecules it does not converge are solved again
    from the core-Hamiltonian guess (the fallback).  Returns (result, fallback indices)."""
    args = [(m["nuc"], m["flat"], m["charge"]) for m in mols]
    D0 = initial_densities(net, mols)
    res = qb.runHartreeFockBatched(args, initial_densities=D0)
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
