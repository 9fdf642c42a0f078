"""One- and two-electron integrals on the GPU against the CPU oracle and the
reference's golden values.  Tolerance: 1e-12 absolute on integrals (the
parity bar of the integral path), unless stated."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _lih(qb, goldens, key, li1s_alpha=None):
    fs = []
    for f in goldens[key]["lih_basis"]["functions"]:
        al = list(f["alphas"])
        if li1s_alpha is not None and f["name"] == "bfLi1":
            al[1] = li1s_alpha
        fs.append(qb.genGaussTypeOrb(f["center"], al, f["coeffs"], f["ijk"], innerRenormalize=True))
    return qb.flatten(fs)


def test_lih_goldens(qb, goldens):
    fb = _lih(qb, goldens, "coulomb")
    n = goldens["coulomb"]["lih_nuclei"]
    V = qb.nucAttractions(["H", "Li"], n["coords"], fb)
    assert np.abs(V.reshape(-1, order="F") - goldens["coulomb"]["lih_V_colmajor"]["values"]).max() < 1e-13
    S = qb.overlaps(_lih(qb, goldens, "overlap", li1s_alpha=2.936200663))
    assert np.abs(S.reshape(-1) - goldens["overlap"]["lih_S_rowmajor"]["values"]).max() < 1e-14


def test_primitive_coulomb_goldens(qb, goldens):
    P = goldens["coulomb"]["prims"]
    g = lambda k: qb.genGaussTypeOrb(P[k]["center"], P[k]["alpha"], P[k]["ijk"])   # unnormalised
    for ob in goldens["coulomb"]["one_body"]:
        a, b = ob["pair"]
        # one nucleus of charge 1 at the point: V = -(a|1/r_C|b)
        v = qb.nucAttraction([1.0], [ob["point"]], g(a), g(b))
        assert v == pytest.approx(-ob["value"], rel=1e-12)
    for tb in goldens["coulomb"]["two_body"]:
        v = qb.elecRepulsion(g(tb["bra"][0]), g(tb["bra"][1]), g(tb["ket"][0]), g(tb["ket"][1]))
        assert v == pytest.approx(tb["value"], rel=1e-11, abs=1e-18)


def test_kinetic_goldens(qb, goldens):
    k = goldens["kinetic"]
    p = qb.genGaussTypeOrb(k["pgto"]["center"], k["pgto"]["alpha"], k["pgto"]["ijk"])
    assert qb.elecKinetic(p, p) == pytest.approx(k["pgto"]["T"], rel=1e-13)
    c = k["cgto"]
    cg = qb.genGaussTypeOrb(c["center"], c["alphas"], c["coeffs"], c["ijk"])
    assert qb.elecKinetic(cg, cg) == pytest.approx(c["T"], rel=1e-12)


@pytest.mark.parametrize("name", ["STO-3G", "6-31G", "cc-pVDZ"])
def test_one_body_matrices_vs_oracle(qb, oracle, name):
    from quiqbox_gb300.workloads import H2O_ATOMS, H2O_BENCH_COORDS, molecule_basis
    fb = qb.flatten(molecule_basis(H2O_ATOMS, H2O_BENCH_COORDS, name))
    nuc = qb.NuclearCluster(H2O_ATOMS, H2O_BENCH_COORDS)
    S = qb.overlaps(fb)
    assert np.abs(S - oracle.overlaps(fb, exact=True)).max() < TOL
    assert np.abs(S - oracle.overlaps(fb)).max() < TOL
    T = qb.elecKinetics(fb)
    assert np.abs(T - oracle.kinetics(fb, exact=True)).max() < TOL
    V = qb.nucAttractions(nuc, fb)
    assert np.abs(V - oracle.nuc_attractions(fb, nuc.charges, nuc.positions, exact=True)).max() < TOL
    H = qb.coreHamiltonian(nuc, fb)
    assert np.array_equal(H, T + V)   # coreHamiltonian == elecKinetics + nucAttractions (Interface-test.jl:58)


def test_eri_tensor_vs_oracle_and_symmetry(qb, oracle):
    from quiqbox_gb300.workloads import H2O_ATOMS, H2O_BENCH_COORDS, molecule_basis
    fb = qb.flatten(molecule_basis(H2O_ATOMS, H2O_BENCH_COORDS, "6-31G"))
    E = qb.elecRepulsions(fb)
    assert np.abs(E - oracle.eri_tensor(fb, exact=True)).max() < TOL
    assert np.abs(E - oracle.eri_tensor(fb)).max() < TOL
    for perm in ((1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1)):
        assert np.array_equal(E, E.transpose(perm))


def test_high_angular_momentum_and_mixed_centres(qb, oracle):
    # primitives of the reference tests with L up to 10 (Coulomb-test.jl:9-17), in contracted
    # functions whose primitives sit on different centres (Framework-test.jl:8-16)
    p1 = qb.genGaussTypeOrb((0.1, 0.2, 0.3), 2.0, (1, 7, 2))
    p2 = qb.genGaussTypeOrb((0.3, 0.1, 0.5), 2.0, (0, 0, 0))
    p3 = qb.genGaussTypeOrb((0.9, 0.6, 0.1), 2.5, (1, 1, 0), renormalize=True)
    p4 = qb.genGaussTypeOrb((0.6, 0.7, 0.8), 3.0, (3, 1, 2))
    c1 = qb.CompositeOrb((p2, p3, p4), (2.0, -1.0, 3.0), renormalize=True)
    bs = [p1, p2, p3, p4, c1]
    fb = qb.flatten(bs)
    assert np.abs(qb.overlaps(fb) - oracle.overlaps(fb, exact=True)).max() < TOL
    assert np.abs(qb.elecKinetics(fb) - oracle.kinetics(fb, exact=True)).max() < TOL
    Z, R = [3.0, 1.0], [(0.0, 0.0, 0.0), (0.4, -0.3, 0.2)]
    assert np.abs(qb.nucAttractions(Z, R, fb) - oracle.nuc_attractions(fb, Z, R, exact=True)).max() < TOL
    q = [(0, 1, 2, 3), (4, 4, 4, 4), (0, 4, 3, 2), (1, 2, 4, 0)]
    g = qb.elecRepulsion_list(fb, q)
    r = oracle.eri_list(fb, q, exact=True)
    assert np.allclose(g, r, rtol=1e-12, atol=TOL)


def test_errors_are_statuses(qb):
    bad = qb.genGaussTypeOrb((0, 0, 0), 1.0, (13, 0, 0))
    with pytest.raises(NotImplementedError):
        qb.overlaps([bad])
    neg = qb.genGaussTypeOrb((0, 0, 0), -1.0)
    with pytest.raises(qb.DomainError):
        qb.overlaps([neg])
    ok = qb.genGaussTypeOrb((0, 0, 0), 1.0)
    with pytest.raises(qb.DimensionMismatch):
        qb.elecRepulsion_list([ok], [(0, 0, 0, 1)])
