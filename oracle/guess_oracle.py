"""CPU restatement of the learned guess's atom-pair features and density assembly (test
infrastructure only: the library computes both on the device, csrc/guess.cu; this float64
numpy version is what the GPU tests compare against).

Pairs (a <= b) of every molecule, their local frames and 128-wide feature rows, and the
inverse map from local-frame 5 x 5 blocks back to per-molecule densities.  The learned
guess has no reference counterpart (the reference's guesses are CoreH / GWH / SAD /
Direct, src/HartreeFock.jl:162-293), so this restatement is its oracle.
"""
import numpy as np

ELEMENTS = ("H", "C", "N", "O")
NBASIS = {"H": 1, "C": 5, "N": 5, "O": 5}
NIN = 128
MU = 0.25 + 0.25 * np.arange(32)


def _unit(v):
    return v / np.maximum(np.linalg.norm(v, axis=-1, keepdims=True), 1e-300)


def atom_offsets(symbols):
    off, o = [], 0
    for s in symbols:
        off.append(o)
        o += NBASIS[s]
    return off, o


def _gather_index(symbols):
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
