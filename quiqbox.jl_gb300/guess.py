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
FALLBACK_ITER = 60      # learned-guess iterations before the core-Hamiltonian restart


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


def pair_index(mols):
    """Host-side index arrays of every atom pair (a <= b) of every molecule: molecule and
    local / global atom indices, atoms' positions, elements and first functions, the
    molecules' sizes and offsets of their column-major densities (vectorised numpy)."""
    code = {e: i for i, e in enumerate(ELEMENTS)}
    nats = np.array([len(m["symbols"]) for m in mols], np.int64)
    nm = len(mols)
    atom0 = np.zeros(nm, np.int64)
    atom0[1:] = np.cumsum(nats)[:-1]
    pos = np.concatenate([np.asarray(m["coords"], np.float64).reshape(-1, 3) for m in mols])
    el = np.array([code[s] for m in mols for s in m["symbols"]], np.int32)
    tri = {n: np.triu_indices(n) for n in np.unique(nats)}
    cnt = nats * (nats + 1) // 2
    pm = np.repeat(np.arange(nm), cnt)
    pa = np.concatenate([tri[n][0] for n in nats]).astype(np.int64)
    pb = np.concatenate([tri[n][1] for n in nats]).astype(np.int64)
    nb = np.where(el == 0, 1, 5)
    fx = np.cumsum(nb) - nb                              # global first function of each atom
    atom_f0 = (fx - np.repeat(fx[atom0], nats)).astype(np.int32)
    mol_n = np.add.reduceat(nb, atom0).astype(np.int32)
    mol_off = np.zeros(nm, np.int64)
    mol_off[1:] = np.cumsum(mol_n.astype(np.int64) ** 2)[:-1]
    return {"mol": pm, "a": pa, "b": pb, "ga": atom0[pm] + pa, "gb": atom0[pm] + pb, "atom0": atom0, "nats": nats,
            "pos": pos, "el": el, "atom_f0": atom_f0, "mol_n": mol_n, "mol_off": mol_off,
            "charge": np.array([m["charge"] for m in mols], np.float32)}


def pair_data(mols, lib, device="cuda:0", host=True):
    """Pairs of every molecule with their local frames and network inputs, computed on the
    device by qb_guess_features (csrc/guess.cu describes the frames and features).
    Returns the index arrays of pair_index plus device tensors "Xd" (rows padded to a
    multiple of 64, zero beyond the pairs) and "Rd"; with host=True also "X" (npair x 128)
    and "R" (npair x 3 x 3, columns the local axes) as numpy arrays."""
    import torch
    pd = pair_index(mols)
    dev = torch.device(device)
    npair = len(pd["mol"])
    M = max(64, ((npair + 63) // 64) * 64)
    t = {k: torch.tensor(pd[k], dtype=torch.int32, device=dev) for k in ("mol", "ga", "gb", "atom0", "nats", "el",
                                                                          "atom_f0", "mol_n")}
    t["pos"] = torch.tensor(pd["pos"], device=dev)
    t["charge"] = torch.tensor(pd["charge"], device=dev)
    t["mol_off"] = torch.tensor(pd["mol_off"], device=dev)
    Xd = torch.zeros((M, NIN), dtype=torch.float32, device=dev)
    Rd = torch.empty((max(npair, 1), 9), dtype=torch.float64, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rc = lib.qb_guess_features(npair, _ptr(t["mol"]), _ptr(t["ga"]), _ptr(t["gb"]), _ptr(t["atom0"]),
                               _ptr(t["nats"]), _ptr(t["pos"]), _ptr(t["el"]), _ptr(t["charge"]), _ptr(Xd),
                               _ptr(Rd), stream)
    if rc != 0:
        raise RuntimeError(f"qb_guess_features failed with status {rc}")
    pd.update({"Xd": Xd, "Rd": Rd, "dev": t, "stream": stream, "npair": npair})
    if host:
        pd["X"] = Xd[:npair].cpu().numpy()
        pd["R"] = Rd[:npair].cpu().numpy().reshape(npair, 3, 3)
    return pd


def assemble_device(lib, pd, Yd):
    """Per-spin initial densities of all molecules (device, column-major, concatenated)
    from the network's output rows Yd (device, one row per pair) by qb_guess_assemble."""
    import torch
    t = pd["dev"]
    total = int(pd["mol_off"][-1] + int(pd["mol_n"][-1]) ** 2) if len(pd["mol_n"]) else 0
    D = torch.zeros(max(total, 1), dtype=torch.float64, device=Yd.device)
    rc = lib.qb_guess_assemble(pd["npair"], _ptr(t["mol"]), _ptr(t["ga"]), _ptr(t["gb"]), _ptr(t["el"]),
                               _ptr(t["atom_f0"]), _ptr(t["mol_off"]), _ptr(t["mol_n"]), _ptr(Yd), Yd.shape[1],
                               _ptr(pd["Rd"]), _ptr(D), pd["stream"])
    if rc != 0:
        raise RuntimeError(f"qb_guess_assemble failed with status {rc}")
    return D


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

    def predict_device(self, Xd):
        """Xd (M, NIN) float32 on the device, M a multiple of 64 -> Y (M, NOUT) on the device."""
        Y, _ = self.forward(self.to_bf16(Xd))
        return Y


def _pad_rows(a, mult=64):
    n = a.shape[0]
    M = ((n + mult - 1) // mult) * mult
    if M == n:
        return a
    out = np.zeros((M,) + a.shape[1:], a.dtype)
    out[:n] = a
    return out


# ---------------------------------------------------------------------------
def dataset(mols, densities, lib=None):
    """Network inputs (device features) and local-frame target blocks with their masks."""
    from . import _lib as L
    pd = pair_data(mols, lib or L.load())
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


def initial_density_device(net, mols):
    """Learned initial per-spin densities of generated molecules, all on the device:
    features, network and assembly; returns the concatenated column-major densities (the
    batched SCF's initial-density layout) as one float64 device tensor."""
    pd = pair_data(mols, net.lib, device=net.dev, host=False)
    return assemble_device(net.lib, pd, net.predict_device(pd["Xd"]))


def initial_densities(net, mols):
    """Learned initial per-spin densities as a list of host matrices."""
    D = initial_density_device(net, mols).cpu().numpy()
    out, off = [], 0
    for m in mols:
        n = m["flat"].nfun
        out.append(D[off:off + n * n].reshape((n, n), order="F"))
        off += n * n
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


def solve_with_guess(qb, net, mols, fallback_iter=FALLBACK_ITER, max_iter=200):
    """Batched SCF from the learned guess in one call; a molecule the learned density has
    not converged after `fallback_iter` iterations restarts from the core-Hamiltonian
    guess inside the same call (0: no fallback), all iterations counted against
    `max_iter`.  Returns (result, indices of the restarted molecules)."""
    args = [(m["nuc"], m["flat"], m["charge"]) for m in mols]
    D0 = initial_density_device(net, mols)
    cfg = qb.BatchSCFConfig(max_iter=max_iter, fallback_iter=fallback_iter)
    res = qb.runHartreeFockBatched(args, config=cfg, initial_densities=D0)
    return res, [int(k) for k in np.nonzero(res.restarted)[0]]


def evaluate(qb, net, n_test=2000, seed=202, fallback_iter=FALLBACK_ITER):
    """Held-out comparison of the core-Hamiltonian and learned guesses (both one batched
    call, at most 200 iterations per molecule)."""
    import torch
    from quiqbox_gb300.workloads import batch_molecules
    mols = batch_molecules(n_test, seed=seed, atoms=(3, 12), basis_names=("STO-3G",))
    args = [(m["nuc"], m["flat"], m["charge"]) for m in mols]
    qb.runHartreeFockBatched(args[:16])   # warm-up of both paths
    solve_with_guess(qb, net, mols[:16], fallback_iter)
    t0 = time.perf_counter()
    base = qb.runHartreeFockBatched(args)
    t_base = time.perf_counter() - t0
    t0 = time.perf_counter()
    lrn, redo = solve_with_guess(qb, net, mols, fallback_iter)
    t_lrn = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    initial_density_device(net, mols)
    torch.cuda.synchronize()
    t_guess = time.perf_counter() - t0
    both = base.converged & lrn.converged
    dE = np.abs(base.energies[both] - lrn.energies[both])
    signed = lrn.energies - base.energies
    same = both & (np.abs(signed) < 1e-8)
    return {"molecules": n_test, "coreh_converged": int(base.converged.sum()),
            "learned_same_state": int(same.sum()),
            "learned_lower_state": int((both & (signed <= -1e-8)).sum()),
            "learned_higher_state": int((both & (signed >= 1e-8)).sum()),
            "learned_same_state_solves_per_s": float(same.sum() / t_lrn),
            "learned_converged": int(lrn.converged.sum()), "fallback_iter": fallback_iter,
            "restarted_from_coreh": len(redo),
            "coreh_mean_iterations": float(base.iterations[both].mean()),
            "learned_mean_iterations": float(lrn.iterations[both].mean()),
            "coreh_median_iterations": float(np.median(base.iterations[both])),
            "learned_median_iterations": float(np.median(lrn.iterations[both])),
            "coreh_wall_s": t_base, "learned_wall_s": t_lrn, "learned_guess_s": t_guess,
            "coreh_ms_scf": base.ms_scf, "learned_ms_scf": lrn.ms_scf,
            "coreh_solves_per_s": float(base.converged.sum() / t_base),
            "learned_solves_per_s": float(lrn.converged.sum() / t_lrn),
            "p99_abs_dE_both_converged": float(np.sort(dE)[int(0.99 * (len(dE) - 1))]) if len(dE) else None,
            "frac_same_state_1e-8": float((dE < 1e-8).mean()) if len(dE) else None}
