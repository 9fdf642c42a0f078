"""GPU Hartree–Fock against the reference goldens and the CPU oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _h2o_test(qb, goldens, name="STO-3G"):
    h = goldens["hartree_fock"]["h2o"]
    bs = []
    for a, x in zip(h["atoms"], h["coords"]):
        bs += qb.genGaussTypeOrbSeq(x, a, name)
    return h, qb.flatten(bs), qb.NuclearCluster(h["atoms"], h["coords"])


def test_h2o_rhf_golden(qb, goldens):
    # HartreeFock-test.jl:92,111-123 (CoreH, (ADIIS, DIIS, EDIIS, DD), thresholds (1e-4, 1e-8, 1e-10, 1e-15))
    h, fb, nuc = _h2o_test(qb, goldens)
    cfg = qb.HFconfig(initial="CoreH", strategy=qb.SCFconfig(("ADIIS", "DIIS", "EDIIS", "DD"),
                                                             (1e-4, 1e-8, 1e-10, 1e-15)))
    r = qb.runHartreeFock(nuc, fb, cfg)
    assert r.converged
    assert abs(r.energy[0] - h["rhf_E_elec"]) < 1e-10
    assert np.abs(r.fock[0].reshape(-1) - h["rhf_fock_rowmajor"]).max() < h["tol"]
    assert np.abs(r.occu[0][0] - h["rhf_orbital_energies"]).max() < h["tol"]
    S = qb.overlaps(fb)
    D = r.density[0]
    assert np.abs(D @ S @ D - D).max() < 1e-10


def test_h2o_uhf_golden(qb, goldens):
    h, fb, nuc = _h2o_test(qb, goldens)
    cfg = qb.HFconfig(type=qb.UOHartreeFock, initial="GWH",
                      strategy=qb.SCFconfig(("ADIIS", "DIIS", "EDIIS", "DD"), (1e-4, 1e-8, 1e-10, 1e-15)))
    r = qb.runHartreeFock(nuc, fb, cfg)
    assert abs(r.energy[0] - h["uhf_E_elec"]) < 1e-10


def test_bench_geometry_rhf_vs_oracle(qb, oracle):
    # H2O, STO-3G, CoreH, DIIS, |dE| <= 1e-10 and RMS(dD) <= 1e-8
    from quiqbox_gb300.workloads import h2o
    nuc, fb = h2o()
    cfg = qb.HFconfig(initial="CoreH", strategy=qb.SCFconfig(("DIIS",), (1e-10,), secondaryConvRatio=(1e6, 100.0)))
    r = qb.runHartreeFock(nuc, fb, cfg)
    ro = oracle.hartree_fock(fb, nuc.charges, nuc.positions, 5, 5, guess="CoreH", methods=("DIIS",),
                             intervals=(1e-10,), secondary=(1e6, 100.0))
    assert r.converged and ro["converged"] == 1
    assert abs(r.energy[0] - ro["E_elec"]) < 1e-10


@pytest.mark.parametrize("guess", ["CoreH", "SAD"])
def test_h2_321g_curve_points(qb, goldens, guess):
    hf = goldens["hartree_fock"]
    for n in (0, 3, 6, 10, 20, 40, 70, 99):
        L = 0.1 + 0.2 * n
        coords = [(0.0, 0.0, 0.0), (L, 0.0, 0.0)]
        bs = qb.genGaussTypeOrbSeq(coords[0], "H", "3-21G") + qb.genGaussTypeOrbSeq(coords[1], "H", "3-21G")
        nuc = qb.NuclearCluster(["H", "H"], coords)
        for typ, ref in ((qb.RCHartreeFock, hf["h2_rhfs"]["values"]), (qb.UOHartreeFock, hf["h2_uhfs"]["values"])):
            r = qb.runHartreeFock(nuc, bs, qb.HFconfig(type=typ, initial=guess, maxStep=300))
            assert abs(sum(r.energy) - ref[n]) < hf["h2_curve"]["tol"], (L, typ)


def test_h2o2_631g_sad(qb, goldens):
    h = goldens["hartree_fock"]["h2o2"]
    coords = [[c * h["angstrom_to_bohr"] for c in x] for x in h["coords_angstrom"]]
    bs = []
    for a, x in zip(h["atoms"], coords):
        bs += qb.genGaussTypeOrbSeq(x, a, "6-31G")
    nuc = qb.NuclearCluster(h["atoms"], coords)
    cfg = qb.HFconfig(strategy=qb.SCFconfig.default(threshold=h["threshold"], secondaryConvRatio=(5.0, 5.0)))
    r = qb.runHartreeFock(nuc, bs, cfg)
    assert r.converged
    assert abs(r.energy[0] - h["E_elec"]) < h["tol"]


def test_dimension_mismatch_of_direct_guess(qb, goldens):
    # HartreeFock-test.jl:46-52: a wrong-size initial coefficient matrix is a DimensionMismatch
    h, fb, nuc = _h2o_test(qb, goldens)
    with pytest.raises(qb.DimensionMismatch):
        qb.runHartreeFock(nuc, fb, qb.HFconfig(initial=(np.zeros((1, 1)),)))
