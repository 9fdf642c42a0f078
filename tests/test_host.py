"""Host-side mirror of the reference's Julia structures (no GPU)."""
import math

import numpy as np
import pytest


def test_basis_sizes(qb):
    # STO-3G: H 1 function, O 5 (1s, 2s, 2p x3); 6-31G: H 2, O 9; cc-pVDZ C: 3s 2p 1d -> 3+6+6
    assert len(qb.genGaussTypeOrbSeq((0, 0, 0), "H", "STO-3G")) == 1
    assert len(qb.genGaussTypeOrbSeq((0, 0, 0), "O", "STO-3G")) == 5
    assert len(qb.genGaussTypeOrbSeq((0, 0, 0), "O", "6-31G")) == 9
    assert len(qb.genGaussTypeOrbSeq((0, 0, 0), "C", "cc-pVDZ")) == 15


def test_missing_basis_is_a_domain_error(qb):
    with pytest.raises(ValueError, match="DomainError"):
        qb.genGaussTypeOrbSeq((0, 0, 0), "K", "cc-pVDZ")


def test_component_order_and_norm_factor(qb):
    # SubshellXYZs (src/Lexicons.jl:17-36)
    assert qb.cartesian_components(2) == [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)]
    # normalised s primitive: (2a/pi)^(3/4)
    a = 0.7
    assert qb.norm_factor(a, (0, 0, 0)) == pytest.approx((2 * a / math.pi) ** 0.75, rel=1e-15)


def test_flatten_weights_bake_normalisation(qb):
    bs = qb.genGaussTypeOrbSeq((0.1, 0.2, 0.3), "O", "STO-3G")
    fb = qb.flatten(bs)
    assert fb.nfun == 5 and list(fb.fun_ptr) == [0, 3, 6, 9, 12, 15]
    assert np.allclose(fb.center, [0.1, 0.2, 0.3])
    px = bs[2]
    w0 = px.effective()[0][1]
    assert w0 == pytest.approx(px.weights[0])   # no renormalisation by default


def test_renormalised_composite_has_unit_norm(qb):
    from quiqbox_gb300.basis import primitive_overlap
    g = qb.genGaussTypeOrb((1.0, 1.5, 1.1), [1.5, 0.6], [1.0, 0.8], (1, 0, 0), outerRenormalize=True)
    eff = g.effective()
    s = sum(wa * wb * primitive_overlap(pa, pb) for pa, wa in eff for pb, wb in eff)
    assert s == pytest.approx(1.0, abs=1e-14)


def test_nuclear_cluster_sorting_and_repulsion(qb):
    nuc = qb.NuclearCluster(["O", "H", "H"], [(0, 0, 0), (0.7, 0, 0), (-0.7, 0, 0)])
    assert nuc.symbols == ["H", "H", "O"] and nuc.coords[0] == (-0.7, 0.0, 0.0)
    enn = qb.nucRepulsion(nuc)
    assert enn == pytest.approx(1 / 1.4 + 2 * 8 / 0.7, rel=1e-15)
    assert qb.prepareSpinConfiguration(nuc) == (5, 5)


def test_workload_generator_shapes(qb):
    from quiqbox_gb300.workloads import random_shell_molecule, random_density
    atoms, coords, bs = random_shell_molecule(seed=1)
    assert len(atoms) == 80 and len(bs) == 64 * 4 + 16 * 10
    c = np.array(coords)
    d = np.linalg.norm(c[:, None] - c[None], axis=-1) + np.eye(len(c)) * 100
    assert d.min() >= 1.3 and c.min() >= 0 and c.max() <= 14
    D = random_density(20)
    assert np.allclose(D, D.T) and np.linalg.eigvalsh(D).min() > -1e-12


def test_batch_molecule_generator():
    # batched-SCF workload: 2-16 atoms, H:C:N:O = 5:3:1:1, bonded chains with bonds in
    # [1.8, 2.9] bohr and angles in [95, 130] degrees, STO-3G or 6-31G, even electrons
    import numpy as np
    import __graft_entry__ as ge
    qb = ge.load_package()
    from quiqbox_gb300.workloads import batch_molecules, _chain_positions
    mols = batch_molecules(64, seed=0)
    assert len(mols) == 64
    for m in mols:
        assert 2 <= len(m["symbols"]) <= 16
        assert m["basis"] in ("STO-3G", "6-31G")
        z = int(round(m["nuc"].charges.sum()))
        assert (z - m["charge"]) % 2 == 0 and m["charge"] in (0, 1)
        assert 1 <= m["flat"].nfun <= 144
    again = batch_molecules(64, seed=0)
    assert all(a["coords"] == b["coords"] and a["basis"] == b["basis"] for a, b in zip(mols, again))
    rng = np.random.default_rng(1)
    P = _chain_positions(10, rng)
    d = np.linalg.norm(P[1:] - P[:-1], axis=1)
    assert (d >= 1.8).all() and (d <= 2.9).all()
    for k in range(1, 9):
        u, v = P[k - 1] - P[k], P[k + 1] - P[k]
        ang = np.degrees(np.arccos(u @ v / np.linalg.norm(u) / np.linalg.norm(v)))
        assert 95.0 - 1e-9 <= ang <= 130.0 + 1e-9


def test_warp_kernel_configs_fit_shared_memory():
    # every generated warp-kernel configuration (per class: owners G, rows S, warps per
    # block, cooperative epilogue) must fit a block's 227 KB of shared memory with its
    # static tables; variant 4 exists for the classes with >= 90 contracted targets
    import importlib.util
    from pathlib import Path
    gen = Path(__file__).resolve().parents[1] / "quiqbox.jl_gb300" / "csrc" / "gen_eri.py"
    spec = importlib.util.spec_from_file_location("gen_eri", gen)
    g = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(g)
    seen4 = 0
    for cls in g.quartet_classes(2):
        cg = g.ClassGen(*cls)
        nt = len(cg.esets) * len(cg.fsets)
        la, lb, lc, ld = cls
        nint = g.ncart(la) * g.ncart(lb) * g.ncart(lc) * g.ncart(ld)
        nab, nf = g.ncart(la) * g.ncart(lb), len(cg.fsets)
        cfgs = g.warp_configs(nt, nint, nab, nf)
        for v, (G, S, rg, pl, coop, wpb) in cfgs.items():
            dyn = wpb * (S * G * (nt | 1) + (nab * nf + nint if coop else 0)) * 8
            # static tables: counts (2 B x 32 per owner), level table, per-owner ints, window
            static = wpb * (G * 32 * 2 + 257 * 4 + 5 * G * 4 + G + (128 * 9 if rg else 9))
            assert dyn + static <= 227 * 1024, (cls, v)
            assert 1 <= G <= 32 and 1 <= S <= 4
            assert coop == (v == 4 and nint >= g.COOP_MIN_NINT)
        assert (4 in cfgs) == (nt >= g.BIG_NT), cls
        seen4 += 4 in cfgs
    assert seen4 >= 8


def test_segmented_kernel_layout():
    # the segmented kernel (variant 5): per class with >= 90 targets, its shared memory
    # (four accumulator rows of emission slots, the HRR buffers, the count tables) fits a
    # block, and the target -> emission-slot table is a one-to-one map into the rows
    import importlib.util
    from pathlib import Path
    gen = Path(__file__).resolve().parents[1] / "quiqbox.jl_gb300" / "csrc" / "gen_eri.py"
    spec = importlib.util.spec_from_file_location("gen_eri", gen)
    g = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(g)
    seen = 0
    for cls in g.quartet_classes(2):
        cg = g.ClassGen(*cls)
        nt = len(cg.esets) * len(cg.fsets)
        assert cg.seg == (nt >= g.SEG_MIN_NT)
        if not cg.seg:
            continue
        cg.generate()
        la, lb, lc, ld = cls
        nint = g.ncart(la) * g.ncart(lb) * g.ncart(lc) * g.ncart(ld)
        nab, nf = g.ncart(la) * g.ncart(lb), len(cg.fsets)
        nr = cg.seg_nbatch * g.SEG_W
        assert sorted(cg.seg_pos) == sorted(set(cg.seg_pos)) and len(cg.seg_pos) == nt
        assert 0 <= min(cg.seg_pos) and max(cg.seg_pos) < nr and nr - nt < g.SEG_W
        wpb = g.seg_warps(cg.seg_nbatch, nab, nf, nint, nt)
        dyn = wpb * (4 * nr + max(nab * nf + max(nint, nt), g.SEG_STAGE)) * 8
        static = wpb * (32 * 16 * 2 + 5 * 32 * 4 + 32)
        assert static <= wpb * g.SEG_STATIC_PER_WARP
        assert dyn + static <= 227 * 1024, cls
        seen += 1
    assert seen >= 6
