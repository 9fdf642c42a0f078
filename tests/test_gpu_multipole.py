"""Multipole moments on the GPU (multipoleMoments, src/Integration/Interface.jl:95)
against the oracle's quad-precision restatement of GaussianOrbitals.jl:184-247, and
the reference test's identities (Interface-test.jl:38-44)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["STO-3G", "6-31G", "cc-pVDZ"])
@pytest.mark.parametrize("center,degrees", [((0.0, 0.0, 0.0), (0, 0, 0)), ((0.3, -0.2, 0.1), (1, 0, 0)),
                                            ((0.0, 0.5, 1.0), (0, 1, 1)), ((1.0, 0.0, 0.0), (2, 2, 2)),
                                            ((-0.4, 0.2, 0.7), (3, 1, 0))])
def test_multipoles_vs_exact_oracle(qb, oracle, name, center, degrees):
    from quiqbox_gb300.workloads import h2o
    _, fb = h2o(name=name)
    M = qb.multipoleMoments(center, degrees, fb)
    Mr = oracle.multipoles(fb, center, degrees, exact=True)
    assert np.abs(M - Mr).max() < 1e-12 * max(1.0, np.abs(Mr).max())


def test_multipole_reference_identities(qb):
    cen1, cen2 = (1.1, 0.5, 1.1), (1.0, 1.5, 1.1)
    cgf1 = qb.genGaussTypeOrb(cen1, [1.2, 0.6], [1.5, -0.3], (1, 0, 0))
    cgf2 = qb.genGaussTypeOrb(cen2, [1.5, 0.6], [1.0, 0.8], (1, 0, 0))
    cgf3 = qb.genGaussTypeOrb(cen1, [1.2, 0.6], [1.5, -0.3], (3, 0, 0))
    assert qb.multipoleMoment(cen1, (0, 0, 0), cgf1, cgf2) == pytest.approx(qb.overlap(cgf1, cgf2), rel=1e-14)
    assert qb.multipoleMoment(cen1, (2, 0, 0), cgf2, cgf1) == pytest.approx(qb.overlap(cgf2, cgf3), rel=1e-13)
    assert qb.multipoleMoment(cen1, (2, 0, 0), cgf1, cgf2) == pytest.approx(qb.overlap(cgf2, cgf3), rel=1e-13)


def test_multipole_rejects_bad_input(qb):
    from quiqbox_gb300.workloads import h2o
    _, fb = h2o()
    with pytest.raises(qb.DomainError):
        qb.multipoleMoments((0.0, 0.0, 0.0), (-1, 0, 0), fb)
