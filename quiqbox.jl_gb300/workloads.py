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


def reduced_shell_molecule(n_h=4, n_heavy=2, seed=3):
    """The ERI + J/K workload's statistics at a size the quad-precision oracle can check in
    full: the same atoms per volume (80 atoms per (14 bohr)^3), minimum distance, shell
    sets, exponent and coefficient ranges, in a cube holding n_h + n_heavy atoms."""
    box = 14.0 * ((n_h + n_heavy) / 80.0) ** (1.0 / 3.0)
    return random_shell_molecule(n_h=n_h, n_heavy=n_heavy, box=box, seed=seed)


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


BATCH_ELEMENTS = ("H", "C", "N", "O")
BATCH_WEIGHTS = (0.5, 0.3, 0.1, 0.1)      # H:C:N:O = 5:3:1:1


def _chain_positions(n_atoms, rng, bond=(1.8, 2.9), angle=(95.0, 130.0), min_nonbonded=1.8, tries=200):
    """A bonded chain: bond lengths uniform in `bond` (bohr), bond angles uniform in
    `angle` (degrees), dihedrals uniform; chains with two non-bonded atoms closer than
    `min_nonbonded` bohr are redrawn."""
    for _ in range(tries):
        pos = [np.zeros(3)]
        if n_atoms > 1:
            pos.append(np.array([rng.uniform(*bond), 0.0, 0.0]))
        for k in range(2, n_atoms):
            b = rng.uniform(*bond)
            th = np.deg2rad(rng.uniform(*angle))
            ph = rng.uniform(0.0, 2.0 * np.pi)
            a, bb = pos[k - 2], pos[k - 1]
            u = bb - a
            u /= np.linalg.norm(u)
            ref = np.array([0.0, 0.0, 1.0]) if abs(u[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
            v = np.cross(u, ref)
            v /= np.linalg.norm(v)
            w = np.cross(u, v)
            # new bond makes angle th with the previous bond at atom k-1
            d = -np.cos(th) * u + np.sin(th) * (np.cos(ph) * v + np.sin(ph) * w)
            pos.append(bb + b * d)
        P = np.array(pos)
        ok = True
        for i in range(n_atoms):
            for j in range(i + 2, n_atoms):
                if np.linalg.norm(P[i] - P[j]) < min_nonbonded:
                    ok = False
                    break
            if not ok:
                break
        if ok:
            return P
    raise RuntimeError("could not place a non-overlapping chain")


def batch_molecules(n_mol=512, seed=0, atoms=(2, 16), basis_names=("STO-3G", "6-31G")):
    """Seeded molecules of the batched-SCF workload: atom count uniform in `atoms`,
    elements H:C:N:O = 5:3:1:1, bonded-chain geometry, basis picked uniformly from
    `basis_names`, charge 0 or +1 so that the electron count is even (closed shell).

    Returns a list of dicts with keys symbols, coords, basis, charge, nuc, flat."""
    from .basis import NUCLEAR_CHARGE
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_mol):
        na = int(rng.integers(atoms[0], atoms[1] + 1))
        syms = [BATCH_ELEMENTS[i] for i in rng.choice(4, size=na, p=BATCH_WEIGHTS)]
        P = _chain_positions(na, rng)
        name = basis_names[int(rng.integers(0, len(basis_names)))]
        zsum = sum(NUCLEAR_CHARGE[s] for s in syms)
        charge = zsum % 2
        coords = [tuple(float(v) for v in p) for p in P]
        nuc = NuclearCluster(syms, coords)
        fb = flatten(molecule_basis(nuc.symbols, nuc.coords, name))
        out.append(dict(symbols=nuc.symbols, coords=nuc.coords, basis=name, charge=charge, nuc=nuc, flat=fb))
    return out
