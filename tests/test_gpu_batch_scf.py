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
    for k, m in enumerate(mols):
        ro = _oracle_rhf(oracle, m)
        assert ro["converged"] == 1
        assert abs(res.elec_energies[k] - ro["E_elec"]) < 1e-10, (k, res.elec_energies[k], ro["E_elec"])


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
    assert (res.iterations[~res.converged] == 200).all()
    small = [k for k in np.where(~res.converged)[0] if mols[k]["flat"].nfun <= 40]
    assert small
    for k in small:
        ro = _oracle_rhf(oracle, mols[k], max_step=200)
        assert ro["converged"] == 0


def test_batched_rhf_rejects_d_shells(qb):
    from quiqbox_gb300.workloads import h2o
    nuc, fb = h2o(name="cc-pVDZ")
    with pytest.raises(Exception):
        qb.runHartreeFockBatched([(nuc, fb)])
