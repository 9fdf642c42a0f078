"""Fused ERI + J/K build (generated HGP class kernels and the generic path)
against the CPU oracle's direct J/K, plus size-independent properties at the
benchmark size."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _small_shell_system(qb, seed, n_h=4, n_heavy=2, box=5.0):
    from quiqbox_gb300.workloads import random_shell_molecule, random_density
    atoms, coords, bs = random_shell_molecule(n_h=n_h, n_heavy=n_heavy, box=box, min_dist=1.0, seed=seed)
    fb = qb.flatten(bs)
    return fb, random_density(fb.nfun, seed)


@pytest.mark.parametrize("seed", [0, 1])
def test_jk_shell_path_vs_exact_oracle(qb, oracle, seed):
    # 2 H (s, p) + 1 heavy atom (s, p, d): every one of the 21 classes occurs.  The
    # reference is evaluated in quad precision (exact); tolerance 1e-12 x max|J|.
    fb, D = _small_shell_system(qb, seed, n_h=2, n_heavy=1, box=4.0)
    J, K = qb.jk(fb, D, schwarz=0.0)
    Jr, Kr = oracle.jk(fb, D, exact=True)
    scale = max(np.abs(Jr).max(), 1.0)
    assert np.abs(J - Jr).max() < 1e-12 * scale
    assert np.abs(K - Kr).max() < 1e-12 * scale


def test_jk_shell_path_vs_reference_float64(qb, oracle):
    # Against the reference's own Float64 algorithm on 36 functions: agreement is limited by
    # that algorithm's electron-transfer round-off (up to ~1e-8 on tight-bra / diffuse-ket
    # quartets), not by the GPU kernels.
    fb, D = _small_shell_system(qb, 0)
    J, K = qb.jk(fb, D, schwarz=0.0)
    Jr, Kr = oracle.jk(fb, D)
    scale = max(np.abs(Jr).max(), 1.0)
    assert np.abs(J - Jr).max() < 1e-8 * scale
    assert np.abs(K - Kr).max() < 1e-8 * scale


def test_jk_generic_path_vs_oracle(qb, oracle):
    # a function whose primitives sit on different centres forces the generic per-function kernels
    fb0, D = _small_shell_system(qb, 3, n_h=3, n_heavy=1, box=4.0)
    extra = qb.CompositeOrb((qb.genGaussTypeOrb((0.5, 0.5, 0.5), 1.2), qb.genGaussTypeOrb((1.0, 0.0, 0.5), 0.8, (0, 1, 0))),
                            (0.7, 0.4))
    from quiqbox_gb300.basis import FlatBasis
    fx = qb.flatten([extra])
    fb = FlatBasis(np.concatenate([fb0.fun_ptr, fb0.fun_ptr[-1] + fx.fun_ptr[1:]]).astype(np.int32),
                   np.concatenate([fb0.center, fx.center]), np.concatenate([fb0.ijk, fx.ijk]).astype(np.int32),
                   np.concatenate([fb0.alpha, fx.alpha]), np.concatenate([fb0.weight, fx.weight]))
    from quiqbox_gb300.workloads import random_density
    D = random_density(fb.nfun, 3)
    J, K = qb.jk(fb, D, schwarz=0.0)
    Jr, Kr = oracle.jk(fb, D, exact=True)
    assert np.abs(J - Jr).max() < 1e-11 and np.abs(K - Kr).max() < 1e-11


def test_jk_matches_stored_tensor_contraction(qb):
    # J_ij = sum (ij|kl) D_kl, K_ij = sum (ik|jl) D_kl from the GPU ERI tensor (getGcore, HartreeFock.jl:305-319)
    from quiqbox_gb300.workloads import H2O_ATOMS, H2O_BENCH_COORDS, molecule_basis, random_density
    fb = qb.flatten(molecule_basis(H2O_ATOMS, H2O_BENCH_COORDS, "cc-pVDZ"))
    D = random_density(fb.nfun, 5)
    E = qb.elecRepulsions(fb)
    J, K = qb.jk(fb, D, schwarz=0.0)
    assert np.abs(J - np.einsum("ijkl,kl->ij", E, D)).max() < 1e-11
    assert np.abs(K - np.einsum("ikjl,kl->ij", E, D)).max() < 1e-11


def test_schwarz_screening_error_is_bounded(qb):
    fb, D = _small_shell_system(qb, 4, n_h=8, n_heavy=2, box=12.0)
    J0, K0 = qb.jk(fb, D, schwarz=0.0)
    J1, K1 = qb.jk(fb, D, schwarz=1e-10)
    assert np.abs(J1 - J0).max() < 1e-7 and np.abs(K1 - K0).max() < 1e-7


def test_schwarz_factors_vs_exact_oracle(qb, oracle):
    # the prepared pair table's Q_ab = sqrt(max |(ab|ab)|) against the quad-precision
    # oracle, on a sparse 12-bohr box where many pairs are distant and diffuse (their
    # (ab|ab) is tiny, but Q_ab Q_cd with a compact cd can still pass the threshold)
    import ctypes as C
    from quiqbox_gb300 import _lib as L
    fb, _ = _small_shell_system(qb, 5, n_h=6, n_heavy=2, box=12.0)
    ctx = qb.Context(0)
    b = L.BasisArgs(fb)
    ctx.check(ctx.lib.qb_jk_prepare(ctx.h, b.ref(), 1e-12))
    npair = C.c_int()
    ctx.check(ctx.lib.qb_jk_pair_table(ctx.h, C.byref(npair), None, None, None, None, None))
    fa, fbb, la, lb = [np.zeros(npair.value, np.int32) for _ in range(4)]
    Q = np.zeros(npair.value)
    ctx.check(ctx.lib.qb_jk_pair_table(ctx.h, C.byref(npair), L.iptr(fa), L.iptr(fbb), L.iptr(la), L.iptr(lb),
                                       L.dptr(Q)))
    quartets, owner = [], []
    for k in range(npair.value):
        na, nb = (la[k] + 1) * (la[k] + 2) // 2, (lb[k] + 1) * (lb[k] + 2) // 2
        for x in range(na):
            for y in range(nb):
                quartets.append((fa[k] + x, fbb[k] + y, fa[k] + x, fbb[k] + y))
                owner.append(k)
    vals = oracle.eri_list(fb, np.array(quartets, np.int32), exact=True)
    Qr = np.zeros(npair.value)
    np.maximum.at(Qr, np.array(owner), np.sqrt(np.abs(vals)))
    assert (Qr < 1e-6).sum() > 10          # the box does have distant, diffuse pairs
    assert np.all(np.abs(Q - Qr) <= 1e-10 * Qr + 1e-15)


def test_benchmark_size_properties(qb):
    # 64 H + 16 heavy atoms, s/p/d, N = 416: symmetry, linearity and positivity of the Coulomb/exchange forms
    from quiqbox_gb300.workloads import random_shell_molecule, random_density
    atoms, coords, bs = random_shell_molecule(seed=0)
    fb = qb.flatten(bs)
    n = fb.nfun
    D1 = random_density(n, 0)
    D2 = random_density(n, 1)
    J1, K1 = qb.jk(fb, D1, schwarz=1e-12)
    J2, K2 = qb.jk(fb, D2, schwarz=1e-12)
    J3, K3 = qb.jk(fb, D1 + D2, schwarz=1e-12)
    assert np.abs(J1 - J1.T).max() < 1e-12 * np.abs(J1).max()
    assert np.abs(K1 - K1.T).max() < 1e-12 * np.abs(K1).max()
    assert np.abs(J3 - J1 - J2).max() < 1e-8 * np.abs(J3).max()
    assert np.abs(K3 - K1 - K2).max() < 1e-8 * np.abs(K3).max()
    assert np.sum(D1 * J1) > 0 and np.sum(D1 * K1) > 0


_VARIANT_SCRIPT = r"""
import sys, numpy as np
import __graft_entry__ as ge
qb = ge.load_package()
from quiqbox_gb300.workloads import random_shell_molecule, random_density
out = {}
for tag, kw in (("classes", dict(n_h=2, n_heavy=1, box=4.0, min_dist=1.0, seed=0)),
                ("long", dict(n_h=1, n_heavy=1, box=3.0, min_dist=1.0, nprim=6, seed=5))):
    atoms, coords, bs = random_shell_molecule(**kw)
    fb = qb.flatten(bs)
    D = random_density(fb.nfun, kw["seed"])
    J, K = qb.jk(fb, D, schwarz=0.0)
    out[tag + "_J"], out[tag + "_K"] = J, K
np.savez(sys.argv[1], **out)
"""


@pytest.mark.parametrize("variant", ["thread", "warp", "2" * 21, "3" * 21, "4" * 21, "5" * 21])
def test_jk_kernel_variants(qb, oracle, tmp_path, variant):
    # Every class-kernel variant (one contracted quartet per thread; the configurations of
    # the warp-cooperative kernel with pooled primitive quartets; "4": its cooperative
    # HRR/digestion epilogue, compiled for the classes of >= 81 integrals; "5": the segmented
    # kernel with reduce-scattered accumulation, compiled for the classes of >= 90 targets),
    # selected per process through QB_JK_VARIANT.  "long" has
    # 6-primitive shells: 36 primitive pairs per shell pair and up to 1296 primitive
    # quartets per contracted quartet, beyond the warp kernel's tabulated counts (32) and
    # its per-pass level window (256).
    import os
    import subprocess
    import sys
    from pathlib import Path
    from quiqbox_gb300.workloads import random_shell_molecule, random_density
    root = Path(__file__).resolve().parents[1]
    out = tmp_path / f"jk_{variant[:6]}.npz"
    env = dict(os.environ, QB_JK_VARIANT=variant)
    subprocess.run([sys.executable, "-c", _VARIANT_SCRIPT, str(out)], cwd=root, env=env, check=True, timeout=600)
    got = np.load(out)
    for tag, kw, exact, tol in (("classes", dict(n_h=2, n_heavy=1, box=4.0, min_dist=1.0, seed=0), True, 1e-12),
                                ("long", dict(n_h=1, n_heavy=1, box=3.0, min_dist=1.0, nprim=6, seed=5), False, 1e-10)):
        atoms, coords, bs = random_shell_molecule(**kw)
        fb = qb.flatten(bs)
        D = random_density(fb.nfun, kw["seed"])
        Jr, Kr = oracle.jk(fb, D, exact=exact)
        scale = max(np.abs(Jr).max(), 1.0)
        assert np.abs(got[tag + "_J"] - Jr).max() < tol * scale, tag
        assert np.abs(got[tag + "_K"] - Kr).max() < tol * scale, tag


def test_jk_autotune_keeps_results(qb, oracle):
    # the autotuner picks a kernel variant per class by timing; J and K stay exact
    fb, D = _small_shell_system(qb, 0, n_h=2, n_heavy=1, box=4.0)
    ctx = qb.Context(0)
    chosen = qb.jk_autotune(fb, D, schwarz=0.0, ctx=ctx)
    assert len(chosen) == 21 and all(0 <= v <= 5 for v in chosen.values())
    J, K = qb.jk(fb, D, schwarz=0.0, ctx=ctx)
    Jr, Kr = oracle.jk(fb, D, exact=True)
    scale = max(np.abs(Jr).max(), 1.0)
    assert np.abs(J - Jr).max() < 1e-12 * scale
    assert np.abs(K - Kr).max() < 1e-12 * scale


def test_class_times_and_fp64_peaks(qb, oracle):
    # the measurement hooks: every class kernel timed alone (positive for the classes with
    # work), J and K unchanged afterwards; both FP64 microbenchmarks report a rate
    import ctypes as C
    from quiqbox_gb300 import _lib as L
    fb, D = _small_shell_system(qb, 1, n_h=2, n_heavy=1, box=4.0)
    ctx = qb.Context(0)
    b = L.BasisArgs(fb)
    Df = np.ascontiguousarray(D.reshape(-1, order="F"))
    ctx.check(ctx.lib.qb_jk_prepare(ctx.h, b.ref(), 0.0))
    ctx.check(ctx.lib.qb_jk_upload_density(ctx.h, L.dptr(Df)))
    ctx.check(ctx.lib.qb_jk_execute(ctx.h))
    st = L.QBJKStats()
    ctx.check(ctx.lib.qb_jk_get_stats(ctx.h, C.byref(st)))
    ms = np.zeros(32, np.float32)
    ctx.check(ctx.lib.qb_jk_class_times(ctx.h, 2, ms.ctypes.data_as(C.POINTER(C.c_float))))
    for c in range(st.nclass):
        assert (ms[c] > 0) == (st.class_quartets[c] > 0), c
    n = fb.nfun
    J, K = np.zeros(n * n), np.zeros(n * n)
    ctx.check(ctx.lib.qb_jk_download(ctx.h, L.dptr(J), L.dptr(K)))
    Jr, Kr = oracle.jk(fb, D, exact=True)
    scale = max(np.abs(Jr).max(), 1.0)
    assert np.abs(J.reshape((n, n), order="F") - Jr).max() < 1e-12 * scale
    assert np.abs(K.reshape((n, n), order="F") - Kr).max() < 1e-12 * scale
    assert 0.1 < qb.fp64_peak(ctx) < 100.0
    assert 0.1 < qb.fp64_dmma_peak(ctx) < 100.0


def test_primitive_threshold_override(qb, oracle, tmp_path):
    # QB_JK_PRIM_EPS=0 evaluates every primitive quartet (no primitive Schwarz screening);
    # J and K stay exact with and without the default screening
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    out = tmp_path / "jk_eps0.npz"
    env = dict(os.environ, QB_JK_PRIM_EPS="0")
    subprocess.run([sys.executable, "-c", _VARIANT_SCRIPT, str(out)], cwd=root, env=env, check=True, timeout=600)
    got = np.load(out)
    from quiqbox_gb300.workloads import random_shell_molecule, random_density
    kw = dict(n_h=2, n_heavy=1, box=4.0, min_dist=1.0, seed=0)
    atoms, coords, bs = random_shell_molecule(**kw)
    fb = qb.flatten(bs)
    D = random_density(fb.nfun, kw["seed"])
    Jr, Kr = oracle.jk(fb, D, exact=True)
    J, K = qb.jk(fb, D, schwarz=0.0)
    scale = max(np.abs(Jr).max(), 1.0)
    for Jx, Kx in ((got["classes_J"], got["classes_K"]), (J, K)):
        assert np.abs(Jx - Jr).max() < 1e-12 * scale
        assert np.abs(Kx - Kr).max() < 1e-12 * scale


# ---------------------------------------------------------------------------
# Parity at the bench workload's own size and screening (64 H + 16 heavy atoms, N = 416,
# Schwarz 1e-12, primitive-quartet screening on): the production class kernels evaluated
# on a stratified sample of the surviving shell quartets against the quad-precision
# oracle on the same quartets, and the full build of a reduced workload with the same
# statistics against the oracle's exact J and K (tests/golden/c1_reduced_jk.json).

def _ncart(L):
    return (L + 1) * (L + 2) // 2


def _pair_table(qb, ctx, fb, D, schwarz):
    import ctypes as C
    from quiqbox_gb300 import _lib as L
    b = L.BasisArgs(fb)
    Df = np.ascontiguousarray(D.reshape(-1, order="F"))
    ctx.check(ctx.lib.qb_jk_prepare(ctx.h, b.ref(), schwarz))
    ctx.check(ctx.lib.qb_jk_upload_density(ctx.h, L.dptr(Df)))
    npair = C.c_int()
    ctx.check(ctx.lib.qb_jk_pair_table(ctx.h, C.byref(npair), None, None, None, None, None))
    arr = [np.zeros(npair.value, np.int32) for _ in range(4)]
    Q = np.zeros(npair.value)
    ctx.check(ctx.lib.qb_jk_pair_table(ctx.h, C.byref(npair), *[L.iptr(a) for a in arr], L.dptr(Q)))
    return b, arr[0], arr[1], arr[2], arr[3], Q


def _stratified_survivors(fa, fb_, la, lb, Q, dmax, thr, rng, fq_budget=5000, min_per_class=8):
    """Canonical surviving shell quartets (global pair indices, bra class >= ket class, ket
    index <= bra index within a class), sampled per class: as many as fq_budget function
    quartets allow, at least min_per_class."""
    pcs = sorted(set(zip(la.tolist(), lb.tolist())), key=lambda t: t[0] * (t[0] + 1) // 2 + t[1])
    idx = {pc: np.where((la == pc[0]) & (lb == pc[1]))[0] for pc in pcs}
    picks, per_class = [], {}
    for x, X in enumerate(pcs):
        for Y in pcs[:x + 1]:
            bi, ki = idx[X], idx[Y]
            cand = []
            for ii, P in enumerate(bi):
                kmax = len(ki) if X != Y else ii + 1
                ok = np.where(Q[P] * Q[ki[:kmax]] * dmax >= thr)[0]
                cand.extend((int(P), int(ki[j])) for j in ok)
            if not cand:
                continue
            fq = _ncart(X[0]) * _ncart(X[1]) * _ncart(Y[0]) * _ncart(Y[1])
            k = min(len(cand), max(min_per_class, fq_budget // fq))
            sel = rng.choice(len(cand), k, replace=False)
            picks.extend(cand[i] for i in sel)
            per_class[X + Y] = k
    return picks, per_class


def _expand_pairs(picks, fa, fb_, la, lb):
    """Shell quartets -> function quartets with the degeneracy weights of the build."""
    q, g = [], []
    for P, R in picks:
        deg = (1.0 if fa[P] == fb_[P] else 2.0) * (1.0 if fa[R] == fb_[R] else 2.0) * (1.0 if P == R else 2.0)
        for a in range(_ncart(la[P])):
            for b in range(_ncart(lb[P])):
                for c in range(_ncart(la[R])):
                    for d in range(_ncart(lb[R])):
                        q.append((fa[P] + a, fb_[P] + b, fa[R] + c, fb_[R] + d))
                        g.append(deg)
    return np.asarray(q, np.int32), np.asarray(g)


def test_bench_workload_quartets_vs_exact_oracle(qb, oracle):
    import ctypes as C
    from quiqbox_gb300 import _lib as L
    from quiqbox_gb300.workloads import random_density, random_shell_molecule
    _, _, bs = random_shell_molecule(seed=0)
    fb = qb.flatten(bs)
    n = fb.nfun
    D = random_density(n, 0)
    ctx = qb.Context(0)
    _, fa, fb_, la, lb, Q = _pair_table(qb, ctx, fb, D, 1e-12)
    rng = np.random.default_rng(2024)
    picks, per_class = _stratified_survivors(fa, fb_, la, lb, Q, float(np.abs(D).max()), 1e-12, rng)
    assert len(per_class) == 21 and len(picks) > 9000
    pq = np.ascontiguousarray(np.asarray(picks, np.int32).reshape(-1))
    J = np.zeros(n * n)
    K = np.zeros(n * n)
    ctx.check(ctx.lib.qb_jk_quartet_list(ctx.h, len(picks), L.iptr(pq), L.dptr(J), L.dptr(K)))
    J = J.reshape((n, n), order="F")
    K = K.reshape((n, n), order="F")
    q, g = _expand_pairs(picks, fa, fb_, la, lb)
    Jp, Kp = oracle.jk_list(fb, q, g, D, 0, exact=True)
    Jx, Kx = (Jp + Jp.T) / 4, (Kp + Kp.T) / 8
    assert np.abs(J - Jx).max() < 1e-12, np.abs(J - Jx).max()
    assert np.abs(K - Kx).max() < 1e-12, np.abs(K - Kx).max()
    ctx.close()


def test_reduced_bench_workload_full_build_vs_exact(qb):
    import json
    from pathlib import Path
    from quiqbox_gb300.basis import FlatBasis
    fx = json.loads((Path(__file__).parent / "golden" / "c1_reduced_jk.json").read_text())
    n = fx["nfun"]
    fb = FlatBasis(np.asarray(fx["fun_ptr"], np.int32), np.asarray(fx["center"]).reshape(-1, 3),
                   np.asarray(fx["ijk"], np.int32).reshape(-1, 3), np.asarray(fx["alpha"]), np.asarray(fx["weight"]))
    D = np.asarray(fx["D_colmajor"]).reshape((n, n), order="F")
    Jx = np.asarray(fx["J_colmajor"]).reshape((n, n), order="F")
    Kx = np.asarray(fx["K_colmajor"]).reshape((n, n), order="F")
    scale = np.abs(Jx).max()
    for thr in (0.0, 1e-12):   # unscreened, and with the bench workload's Schwarz threshold
        J, K = qb.jk(fb, D, schwarz=thr)
        assert np.abs(J - Jx).max() < 1e-12 * scale, (thr, np.abs(J - Jx).max())
        assert np.abs(K - Kx).max() < 1e-12 * scale, (thr, np.abs(K - Kx).max())
