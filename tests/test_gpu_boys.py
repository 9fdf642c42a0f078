"""Device Boys function F_m(T) (both evaluators: the one inlined in the ERI class
kernels and the runtime-order one of the generic kernels) against the oracle's
quad-precision restatement of computeBoysSequence
(src/Integration/Engines/BoysFunction.jl:67-77)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid():
    rng = np.random.default_rng(11)
    T = [0.0, 1e-300, 1e-16, 1e-12, 1e-6, 1e-3, 0.03125, 0.0625, 1.0, 10.0, 49.96875, 49.999999,
         50.0, 50.000001, 51.0, 80.0, 100.0, 1e3, 1e5]
    T += list(rng.uniform(0.0, 60.0, 150)) + list(np.exp(rng.uniform(np.log(60.0), np.log(1e4), 30)))
    return np.array(T)


@pytest.mark.parametrize("path,M,rtol", [(0, 8, 2e-14), (1, 32, 5e-14)])
def test_device_boys_vs_exact(qb, oracle, path, M, rtol):
    T = _grid()
    F = qb.computeBoysSequence(T, M, path=path)
    worst = 0.0
    for i, x in enumerate(T):
        for m in range(M + 1):
            ref = oracle.boys_exact(x, m)
            err = abs(F[i, m] - ref) / abs(ref)
            worst = max(worst, err)
            assert err < rtol, (x, m, F[i, m], ref)
    assert worst < rtol


def test_device_boys_goldens(qb, goldens):
    # the reference's own Boys test points (test/unit-tests/Integration/BoysFunction-test.jl:6-31)
    # with orders the device evaluators cover (n <= 32), at the reference tests' rtol sqrt(eps)
    pts = [p for p in goldens["boys"]["points"] if p["n"] <= 32]
    assert len(pts) == 7
    for p in pts:
        got = qb.computeBoysFunc(p["x"], p["n"])
        assert got == pytest.approx(p["F"], rel=1.4901161193847656e-08)


def test_device_boys_rejects_bad_input(qb):
    with pytest.raises(qb.DomainError):
        qb.computeBoysSequence(np.array([-1.0]), 2)
    with pytest.raises(qb.DimensionMismatch):
        qb.computeBoysSequence(np.array([1.0]), 9, path=0)
