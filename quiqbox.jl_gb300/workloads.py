"""Seeded synthetic workloads of the benchmark and the tests.

No public dataset is involved: every input is generated from a seed with the
shapes the benchmark names.
"""
from __future__ import annotations

import numpy as np

from .basis import CompositeOrb, NuclearCluster, PrimitiveOrb, cartesian_components, flatten, genGaussTypeOrbSeq, \
    norm_factor


def random_shell_molecule(n_h=64, n_heavy=16, box=14.0, min_dist=1.3, heavy=("C", "N", "O"),
                          h_shells=(0, 1), heavy_shells=(0, 1, 2), nprim=3, alpha_range=(0.1, 60.0),
                          coef_range=(0.1, 1.0), seed=0):
    """ERI + J/K workload: n_h H and n_heavy atoms (type uniform over `heavy`) placed
    uniformly in a cube of side `box` bohr with no pair closer than `min_dist`;
    per atom one contracted Cartesian shell of each angular momentum in
    h_shells / heavy_shells, `nprim` primitives with exponents log-uniform in
    alpha_range and coefficients uniform in coef_range, normalised per primitive
    as genGaussTypeOrbSeq does (coefficient x get3DimPGTOrbNormFactor).

    Returns (atoms, coords, basis list)."""
    rng = np.random.default_rng(seed)
    atoms = ["H"] * n_h + [heavy[i] for i in rng.integers(0, len(heavy), n_heavy)]
    coords = []
    while len(coords) < len(atoms):
        x = rng.uniform(0.0, box, 3)
        if all(np.linalg.norm(x - c) >= min_dist for c in coords):
            coords.append(x)
    basis = []
    lo, hi = np.log(alpha_range[0]), np.log(alpha_range[1])
    for a, x in zip(atoms, coords):
        for L in (h_shells if a == "H" else heavy_shells):
            al = np.exp(rng.uniform(lo, hi, nprim))
            co = rng.uniform(coef_range[0], coef_range[1], nprim)
            for ijk in cartesian_components(L):
                prims = tuple(PrimitiveOrb(tuple(float(v) for v in x), float(e), ijk) for e in al)
                w = tuple(float(c * norm_factor(e, ijk)) for c, e in zip(co, al))
                basis.append(CompositeOrb(prims, w))
    return atoms, [tuple(float(v) for v in c) for c in coords], basis


def random_density(n, seed=0):
    """Symmetric positive semidefinite D = A A^T / n, A uniform in [-1, 1]."""
    rng = np.random.default_rng(seed + 7919)
    A = rng.uniform(-1.0, 1.0, (n, n))
    return A @ A.T / n


def molecule_basis(atoms, coords, name):
    bs = []
    for a, x in zip(atoms, coords):
        bs += genGaussTypeOrbSeq(x, a, name)
    return bs


H2O_ATOMS = ["H", "H", "O"]
H2O_TEST_COORDS = [(-0.7, 0.0, 0.0), (0.7, 0.0, 0.0), (0.0, 0.0, 0.0)]     # HartreeFock-test.jl:12
H2O_BENCH_COORDS = [(0.0, 1.4305, 1.1093), (0.0, -1.4305, 1.1093), (0.0, 0.0, 0.0)]


def h2o(coords=H2O_BENCH_COORDS, name="STO-3G"):
    return NuclearCluster(H2O_ATOMS, coords), flatten(molecule_basis(H2O_ATOMS, coords, name))
