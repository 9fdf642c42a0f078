"""The learned-guess MLP's CPU oracle (float64, no rounding) against central finite
differences, and the guess's pair-block bookkeeping (features, local frames, assembly)."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import mlp_oracle as mo  # noqa: E402


def _params(rng, dims):
    p = {}
    for l in range(len(dims) - 1):
        p["W%d" % l] = rng.normal(0, 0.5, (dims[l + 1], dims[l]))
        p["b%d" % l] = rng.normal(0, 0.1, dims[l + 1])
    return p


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    dims = [6, 5, 5, 4]
    p = _params(rng, dims)
    X = rng.normal(size=(7, 6))
    T = rng.normal(size=(7, 4))
    W = (rng.uniform(size=(7, 4)) > 0.3).astype(float)

    def loss(pp):
        Y, _ = mo.forward(pp, X, round=False)
        return mo.mse(Y, T, W)[0]

    Y, saved = mo.forward(p, X, round=False)
    _, dY = mo.mse(Y, T, W)
    dW, db = mo.backward(p, saved, dY, round=False)
    h = 1e-6
    for l in range(3):
        for name, g in (("W%d" % l, dW[l]), ("b%d" % l, db[l])):
            flat = p[name].reshape(-1)
            for idx in range(0, flat.size, max(1, flat.size // 7)):
                old = flat[idx]
                flat[idx] = old + h
                lp = loss(p)
                flat[idx] = old - h
                lm = loss(p)
                flat[idx] = old
                assert g.reshape(-1)[idx] == pytest.approx((lp - lm) / (2 * h), rel=1e-5, abs=1e-9)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.0078125, 3.14159265, -2.5e-3], np.float64)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0          # halfway: ties to even
    assert r[2] == 1.0078125                    # representable
    assert abs(r[3] - 3.140625) < 1e-12
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)


def test_guess_blocks_round_trip():
    # the oracle's features and assembly with the library's host-side target blocks
    import __graft_entry__ as ge
    ge.load_package()
    import guess_oracle as go
    from quiqbox_gb300 import guess
    from quiqbox_gb300.workloads import batch_molecules
    mols = batch_molecules(12, seed=9, atoms=(2, 10), basis_names=("STO-3G",))
    pd = go.pair_data(mols)
    rng = np.random.default_rng(1)
    dens = []
    for m in mols:
        _, n = guess.atom_offsets(m["symbols"])
        assert n == m["flat"].nfun
        A = rng.normal(size=(n, n))
        dens.append(A + A.T)
    Y, W = guess.blocks_from_densities(mols, dens, pd)
    D2 = go.densities_from_blocks(mols, pd, Y)
    assert max(np.abs(a - b).max() for a, b in zip(dens, D2)) < 1e-5
    R = pd["R"]
    assert np.abs(np.einsum("pij,pik->pjk", R, R) - np.eye(3)).max() < 1e-12
    assert np.abs(np.linalg.det(R) - 1.0).max() < 1e-12
    assert pd["X"].shape == (len(pd["mol"]), guess.NIN) and np.isfinite(pd["X"]).all()
    # rotating and translating every molecule leaves the features and the local-frame
    # blocks of the rotated densities unchanged
    Q = np.linalg.qr(rng.normal(size=(3, 3)))[0]
    if np.linalg.det(Q) < 0:
        Q[:, 0] *= -1
    rot = []
    for m in mols:
        m2 = dict(m)
        m2["coords"] = [tuple(Q @ np.array(c) + 1.5) for c in m["coords"]]
        rot.append(m2)
    pd2 = go.pair_data(rot)
    assert np.abs(pd2["X"] - pd["X"]).max() < 1e-5
    dens2 = []
    for m, D in zip(mols, dens):
        T = np.eye(len(D))
        off, _ = guess.atom_offsets(m["symbols"])
        for i, s in enumerate(m["symbols"]):
            if guess.NBASIS[s] == 5:
                T[off[i] + 2:off[i] + 5, off[i] + 2:off[i] + 5] = Q
        dens2.append(T @ D @ T.T)
    Y2, _ = guess.blocks_from_densities(rot, dens2, pd2)
    assert np.abs(Y2 - Y).max() < 1e-5
