"""Batched closed-shell HF (many molecules per call) against the oracle's restatement
of runHartreeFock (src/HartreeFock.jl:953-1046) run molecule by molecule."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_rhf(oracle, mol, max_step=300):
    # the batched path extrapolates with the exact Pulay coefficients, the solution the
    # Lagrange-multiplier solver gives (CMsolver!, HartreeFock.jl:1445-1477)
    fb, nuc = mol["flat"], mol["nuc"]
    nocc = (int(round(nuc.charges.sum())) - mol["charge"]) // 2
    return oracle.hartree_fock(fb, nuc.charges, nuc.positions, nocc, nocc, guess="CoreH", methods=("DIIS",),
                               intervals=(1e-10,), secondary=(1e6, 100.0), max_step=max_step, solvers=("LCM",))


def test_batched_rhf_vs_oracle(qb, oracle):
    # 20 chains of 2-6 atoms, STO-3G and 6-31G mixed, neutral or +1: every converged
    # electronic energy equals the oracle's to 1e-10 Ha
    from quiqbox_gb300.workloads import batch_molecules
    mols = batch_molecules(20, seed=3, atoms=(2, 6))
    res = qb.runHartreeFockBatched([(m["nuc"], m["flat"], m["charge"]) for m in mols])
    assert res.converged.all(), res.iterations
    assert res.graph_launches == 1   # every iteration of every molecule in one graph launch
    assert res.digest_chunk in (1024, 2048, 4096)   # chosen by timing on this batch
    steps = []
    for k, m in enumerate(mols):
        ro = _oracle_rhf(oracle, m)
        assert ro["converged"] == 1
        assert abs(res.elec_energies[k] - ro["E_elec"]) < 1e-10, (k, res.elec_energies[k], ro["E_elec"])
        steps.append(ro["steps"])
    # the subspace reset on an energy rise above 4e-13 Ha (HartreeFock.jl:1337,1367) makes the
    # last steps' trajectory depend on rounding: iteration counts agree on average
    assert abs(res.iterations.mean() - np.mean(steps)) < 0.15 * np.mean(steps), (res.iterations, steps)


def _oracle_default(oracle, mol, thr=1e-10):
    fb, nuc = mol["flat"], mol["nuc"]
    nocc = (int(round(nuc.charges.sum())) - mol["charge"]) // 2
    return oracle.hartree_fock(fb, nuc.charges, nuc.positions, nocc, nocc, guess="CoreH",
                               methods=("DD", "ADIIS", "DIIS"), intervals=(5e-3, 1e-4, thr),
                               secondary=(1000.0, 1000.0), max_step=200)


def test_batched_default_strategy_vs_oracle(qb, oracle):
    # the reference's default SCFconfig (DD, ADIIS, DIIS) with L-BFGS-B coefficients
    # (HartreeFock.jl:17,27) from the core-Hamiltonian guess, molecule by molecule in the oracle
    from quiqbox_gb300.workloads import batch_molecules
    mols = batch_molecules(24, seed=3, atoms=(2, 6))
    cfg = qb.BatchSCFConfig(strategy=qb.SCFconfig.default(threshold=1e-10))
    res = qb.runHartreeFockBatched([(m["nuc"], m["flat"], m["charge"]) for m in mols], config=cfg)
    assert res.graph_launches == 1
    same_flag, both = 0, 0
    for k, m in enumerate(mols):
        ro = _oracle_default(oracle, m)
        same_flag += bool(res.converged[k]) == (ro["converged"] == 1)
        if ro["converged"] == 1 and res.converged[k]:
            assert abs(res.elec_energies[k] - ro["E_elec"]) < 1e-9, (k, res.elec_energies[k], ro["E_elec"])
            both += 1
    # the L-BFGS-B coefficients stop on tiny objective changes (factr 1e5), so rounding can
    # move a marginal molecule's trajectory; nearly all agree
    assert same_flag >= len(mols) - 1 and both >= 0.75 * len(mols)


def test_batched_default_strategy_matches_single_molecule_path(qb):
    from quiqbox_gb300.workloads import batch_molecules
    mols = [m for m in batch_molecules(12, seed=7, atoms=(2, 7)) if m["charge"] == 0][:5]
    strategy = qb.SCFconfig.default(threshold=1e-10)
    res = qb.runHartreeFockBatched([(m["nuc"], m["flat"]) for m in mols], config=qb.BatchSCFConfig(strategy=strategy))
    for k, m in enumerate(mols):
        r = qb.runHartreeFock(m["nuc"], m["flat"], qb.HFconfig(initial="CoreH", strategy=strategy))
        assert bool(r.converged) == bool(res.converged[k])
        if r.converged:
            # (iteration counts may differ: L-BFGS-B stops on objective changes near rounding,
            # so the two paths' trajectories drift apart in long runs; 57 against 96 steps seen)
            assert abs(res.elec_energies[k] - r.energy[0]) < 1e-9


def test_batched_rhf_matches_single_molecule_path(qb):
    # the same molecules one at a time through runHartreeFock (CoreH, DIIS) on the GPU
    from quiqbox_gb300.workloads import batch_molecules
    mols = [m for m in batch_molecules(12, seed=5, atoms=(2, 8)) if m["charge"] == 0][:6]
    res = qb.runHartreeFockBatched([(m["nuc"], m["flat"]) for m in mols])
    cfg = qb.HFconfig(initial="CoreH", strategy=qb.SCFconfig(("DIIS",), (1e-10,), {1: [("solver", "LCM")]},
                                                             secondaryConvRatio=(1e6, 100.0)), maxStep=300)
    for k, m in enumerate(mols):
        r = qb.runHartreeFock(m["nuc"], m["flat"], cfg)
        assert r.converged
        assert abs(res.elec_energies[k] - r.energy[0]) < 1e-10


def test_batched_rhf_fixed_digest_chunk(qb):
    # a caller-fixed digest chunk (qb_batch_config.digest_chunk) changes only how the stored
    # quartets are split into blocks: same converged energies as the timed choice
    from quiqbox_gb300.workloads import batch_molecules
    mols = batch_molecules(16, seed=9, atoms=(2, 8))
    args = [(m["nuc"], m["flat"], m["charge"]) for m in mols]
    auto = qb.runHartreeFockBatched(args)
    fixed = qb.runHartreeFockBatched(args, config=qb.BatchSCFConfig(digest_chunk=256))
    assert fixed.digest_chunk == 256
    both = auto.converged & fixed.converged
    assert both.sum() >= 12
    assert np.abs(auto.elec_energies[both] - fixed.elec_energies[both]).max() < 1e-10
    with pytest.raises(Exception):
        qb.runHartreeFockBatched(args[:2], config=qb.BatchSCFConfig(digest_chunk=-1))


def test_batched_rhf_full_workload_sizes(qb, oracle):
    # the benchmark's molecule generator at full size range (2-16 atoms, 2-120 functions).
    # Pure DIIS from the core-Hamiltonian guess does not converge every random chain in 200
    # steps; the reference's own algorithm (the oracle) fails on the same molecules, which
    # is checked for the small ones.
    from quiqbox_gb300.workloads import batch_molecules
    mols = batch_molecules(64, seed=0)
    res = qb.runHartreeFockBatched([(m["nuc"], m["flat"], m["charge"]) for m in mols])
    assert np.isfinite(res.energies).all()
    assert res.converged.mean() >= 0.85
    assert res.quartets > 0 and res.eri_doubles > 0
    assert (res.elec_energies < 0).all()
    assert (res.iterations <= 200).all()
    small = [k for k in np.where(~res.converged)[0] if mols[k]["flat"].nfun <= 40]
    assert small
    for k in small:   # the early-stop rule may end a failing molecule before 200 steps
        ro = _oracle_rhf(oracle, mols[k], max_step=200)
        assert ro["converged"] == 0


def test_batched_rhf_rejects_d_shells(qb):
    from quiqbox_gb300.workloads import h2o
    nuc, fb = h2o(name="cc-pVDZ")
    with pytest.raises(Exception):
        qb.runHartreeFockBatched([(nuc, fb)])
