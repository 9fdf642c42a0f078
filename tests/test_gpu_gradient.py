"""Adjoint RHF energy gradient with respect to basis exponents, coefficients and
centres (basis-set optimisation workload: H4 chain and H2O, 2 floating s + 1 p shells
per atom) against central finite differences (h = 1e-5) of the converged energy, to
1e-7 — on the GPU SCF and, for a sample of parameters, on the oracle's restatement of
runHartreeFock.  The reference has no analytic gradient to compare with."""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
H = 1e-5


def _params(shells):
    out = []
    for s, sh in enumerate(shells):
        for k in range(len(sh.exponents)):
            out.append(("exp", s, k))
            out.append(("coef", s, k))
        for ax in range(3):
            out.append(("cen", s, ax))
    return out


def _shift(shells, p, d):
    sh = copy.deepcopy(shells)
    kind, s, k = p
    if kind == "exp":
        sh[s].exponents[k] += d
    elif kind == "coef":
        sh[s].coefficients[k] += d
    else:
        c = list(sh[s].center)
        c[k] += d
        sh[s].center = tuple(c)
    return sh


def _analytic(g, p):
    kind, s, k = p
    return {"exp": g.d_exponents, "coef": g.d_coefficients}[kind][s][k] if kind != "cen" else g.d_centers[s, k]


@pytest.mark.parametrize("system", [0, 1])
def test_gradient_vs_finite_differences_gpu(qb, system):
    from quiqbox_gb300.differentiation import config3_systems, rhf_energy, rhf_energy_gradient
    nuc, shells = config3_systems(seed=0)[system]
    g = rhf_energy_gradient(nuc, shells)
    assert abs(g.energy - rhf_energy(nuc, shells)) < 1e-10
    worst = 0.0
    for p in _params(shells):
        fd = (rhf_energy(nuc, _shift(shells, p, H)) - rhf_energy(nuc, _shift(shells, p, -H))) / (2 * H)
        worst = max(worst, abs(fd - _analytic(g, p)))
        assert abs(fd - _analytic(g, p)) < 1e-7, (p, fd, _analytic(g, p))
    assert worst < 1e-7


def test_gradient_vs_oracle_finite_differences(qb, oracle):
    from quiqbox_gb300.differentiation import config3_systems, rhf_energy_gradient, shells_basis
    nuc, shells = config3_systems(seed=0)[1]
    g = rhf_energy_gradient(nuc, shells)
    nocc = int(round(nuc.charges.sum())) // 2

    def e_oracle(sh):
        r = oracle.hartree_fock(shells_basis(sh), nuc.charges, nuc.positions, nocc, nocc, guess="CoreH",
                                methods=("DIIS",), intervals=(1e-12,), secondary=(1e6, 100.0), max_step=500,
                                solvers=("LCM",))
        assert r["converged"] == 1
        return r["E_elec"] + qb.nucRepulsion(nuc)

    assert abs(e_oracle(shells) - g.energy) < 1e-9
    rng = np.random.default_rng(5)
    ps = _params(shells)
    for i in rng.choice(len(ps), 8, replace=False):
        p = ps[i]
        fd = (e_oracle(_shift(shells, p, H)) - e_oracle(_shift(shells, p, -H))) / (2 * H)
        assert abs(fd - _analytic(g, p)) < 1e-7, (p, fd, _analytic(g, p))
