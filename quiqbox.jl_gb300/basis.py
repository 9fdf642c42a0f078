"""Orbital containers and basis construction, mirroring Quiqbox.jl's Julia side.

This module is the host-side mirror of what stays in Julia in the drop-in:
primitive / contracted Cartesian GTOs (src/OrbitalBases.jl:12-96), their
constructors ``genGaussTypeOrb`` (:199-247) and ``genGaussTypeOrbSeq``
(:502-594), nuclear geometries (``NuclearCluster``, src/Particles.jl:19-51) and
the flattening of a basis into per-primitive arrays with effective weights
(``buildOrbCoreWeight!``, src/Integration/Framework.jl:748-773), which is the
data that crosses the C-ABI boundary (``qb_basis`` in include/quiqbox_gb300.h).
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from pathlib import Path
from typing import Sequence

import numpy as np

# src/Lexicons.jl:10-13
ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne",
            "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar", "K", "Ca"]
NUCLEAR_CHARGE = {s: i + 1 for i, s in enumerate(ELEMENTS)}
# AngularSubShellDict (src/Lexicons.jl:39-46)
SUBSHELL_L = {"S": 0, "P": 1, "D": 2, "F": 3, "G": 4, "H": 5, "I": 6}


def cartesian_components(L: int):
    """SubshellXYZs[L] (src/Lexicons.jl:17-36): x-power descending, then y."""
    return [(i, j, L - i - j) for i in range(L, -1, -1) for j in range(L - i, -1, -1)]


def norm_factor(alpha: float, ijk: Sequence[int]) -> float:
    """get3DimPGTOrbNormFactor (src/OrbitalBases.jl:476-485)."""
    i, j, k = ijk
    L = i + j + k
    f = math.factorial
    ang = (math.pi ** -0.75) * 2.0 ** (1.5 * L + 0.75) * math.sqrt(
        f(i) * f(j) * f(k) / (f(2 * i) * f(2 * j) * f(2 * k)))
    return alpha ** ((2 * L + 3) * 0.25) * ang


def _axial_factor(xsum: float, degree: int) -> float:
    """computePGTOrbOverlapAxialFactor (GaussianOrbitals.jl:94-97)."""
    f = 1.0
    c = 1.0 / (2 * xsum)
    for i in range(1, 2 * degree, 2):
        f *= i * c
    return math.sqrt(math.pi) / math.sqrt(xsum) * f


def _axial_overlap(xsum, xpos, xml, xmr, il, ir):
    """computeAxialPGTOrbOverlap, adaptive (GaussianOrbitals.jl:110-138)."""
    dx = xmr - xml
    if il == 0 and ir == 0:
        return _axial_factor(xsum, 0) * math.exp(-xpos * dx * dx)
    if dx == 0.0:
        return _axial_factor(xsum, (il + ir) // 2) if (il + ir) % 2 == 0 else 0.0
    res = 0.0
    for j in range((il + ir) // 2 + 1):
        lx = 2 * j
        lb, ub = max(-lx, lx - 2 * ir), min(lx, 2 * il - lx)
        gp = 0.0
        for q in range(lb, ub + 1, 2):
            a, b = (lx + q) >> 1, (lx - q) >> 1
            gp += math.comb(il, a) * math.comb(ir, b) * xml ** (il - a) * xmr ** (ir - b)
        res += gp * _axial_factor(xsum, j)
    return res * math.exp(-xpos * dx * dx)


def primitive_overlap(p: "PrimitiveOrb", q: "PrimitiveOrb") -> float:
    """Overlap of two unnormalised primitives (GaussianOrbitals.jl:147-179)."""
    if p.center == q.center and p.alpha == q.alpha and p.ijk == q.ijk:
        r = 1.0
        for l in p.ijk:
            r *= _axial_factor(2 * p.alpha, l)
        return r
    s = p.alpha + q.alpha
    pos = p.alpha * q.alpha / s
    r = 1.0
    for k in range(3):
        m = (p.alpha * p.center[k] + q.alpha * q.center[k]) / s
        r *= _axial_overlap(s, pos, m - p.center[k], m - q.center[k], p.ijk[k], q.ijk[k])
    return r


@dataclass(frozen=True)
class PrimitiveOrb:
    """Primitive Cartesian GTO (x-Ax)^i (y-Ay)^j (z-Az)^k exp(-alpha r^2) (OrbitalBases.jl:12-23)."""
    center: tuple
    alpha: float
    ijk: tuple = (0, 0, 0)
    renormalize: bool = False

    def weight(self) -> float:
        """buildOrbCoreWeight! for a primitive pointer (Framework.jl:748-756)."""
        return 1.0 / math.sqrt(abs(primitive_overlap(self, self))) if self.renormalize else 1.0


@dataclass(frozen=True)
class CompositeOrb:
    """Linear combination of primitives (OrbitalBases.jl:57-96)."""
    basis: tuple
    weights: tuple
    renormalize: bool = False

    def effective(self):
        """Primitive list with effective weights (buildOrbCoreWeight!, Framework.jl:758-773,
        with the composite self-overlap of getOrbCoreOverlap!, :710-745)."""
        w = [c * p.weight() for p, c in zip(self.basis, self.weights)]
        if self.renormalize:
            tot = 0.0
            for p, c, wn in zip(self.basis, self.weights, w):
                tot += c * c if p.renormalize else c * c * primitive_overlap(p, p)
            for a in range(len(w)):
                for b in range(a + 1, len(w)):
                    off = primitive_overlap(self.basis[a], self.basis[b]) * w[a] * w[b]
                    tot += 2 * off
            s = 1.0 / math.sqrt(abs(tot))
            w = [x * s for x in w]
        return list(zip(self.basis, w))


def genGaussTypeOrb(center, xpn, *args, ijk=None, renormalize=False,
                    innerRenormalize=False, outerRenormalize=False):
    """genGaussTypeOrb (OrbitalBases.jl:199-247).

    genGaussTypeOrb(center, alpha[, ijk]; renormalize) -> PrimitiveOrb
    genGaussTypeOrb(center, alphas, coeffs[, ijk]; innerRenormalize, outerRenormalize) -> CompositeOrb
    """
    center = tuple(float(c) for c in center)
    if np.ndim(xpn) == 0:
        ang = tuple(args[0]) if args else (tuple(ijk) if ijk is not None else (0, 0, 0))
        return PrimitiveOrb(center, float(xpn), tuple(int(v) for v in ang), bool(renormalize))
    cons = [float(c) for c in args[0]]
    ang = tuple(args[1]) if len(args) > 1 else (tuple(ijk) if ijk is not None else (0, 0, 0))
    if len(cons) != len(xpn):
        raise ValueError("`xpns` and `cons` must have the same length")
    prims = tuple(PrimitiveOrb(center, float(a), tuple(int(v) for v in ang), innerRenormalize)
                  for a in xpn)
    return CompositeOrb(prims, tuple(cons), bool(outerRenormalize))


_BASIS_SETS = None


def _basis_sets():
    global _BASIS_SETS
    if _BASIS_SETS is None:
        _BASIS_SETS = json.loads((Path(__file__).parent / "data" / "basis_sets.json").read_text())
    return _BASIS_SETS


def basis_set_names():
    return list(_basis_sets().keys())


def genGaussTypeOrbSeq(center, atm: str, basisKey: str, innerRenormalize=False,
                       outerRenormalize=False):
    """genGaussTypeOrbSeq (OrbitalBases.jl:502-594): contracted Cartesian GTOs of an atom.

    Contraction coefficients are multiplied by get3DimPGTOrbNormFactor of each
    primitive; SP subshells expand to L=0 then L=1; components follow SubshellXYZs.
    """
    fam = _basis_sets().get(basisKey)
    if fam is None or atm not in fam:
        raise ValueError(f"DomainError: no pre-stored basis set for ({atm}, {basisKey})")
    out = []
    for sh in fam[atm]:
        Ls = (0, 1) if sh["shell"] == "SP" else (SUBSHELL_L[sh["shell"]],)
        for row, L in enumerate(Ls):
            for ijk in cartesian_components(L):
                cons = [c * norm_factor(a, ijk) for a, c in zip(sh["exponents"], sh["coefficients"][row])]
                out.append(genGaussTypeOrb(center, sh["exponents"], cons, ijk,
                                           innerRenormalize=innerRenormalize,
                                           outerRenormalize=outerRenormalize))
    return out


@dataclass
class NuclearCluster:
    """Nuclear geometry sorted by (charge, coordinates) (src/Particles.jl:19-51)."""
    symbols: list
    coords: list
    pairwiseSort: bool = True

    def __post_init__(self):
        if len(self.symbols) != len(self.coords) or not self.symbols:
            raise ValueError("`nucSyms` and `nucCoords` should have the same non-zero length.")
        order = list(range(len(self.symbols)))
        if self.pairwiseSort:
            order.sort(key=lambda i: (NUCLEAR_CHARGE[self.symbols[i]], tuple(self.coords[i])))
        self.symbols = [self.symbols[i] for i in order]
        self.coords = [tuple(float(c) for c in self.coords[i]) for i in order]

    @property
    def charges(self):
        return np.array([NUCLEAR_CHARGE[s] for s in self.symbols], dtype=np.float64)

    @property
    def positions(self):
        return np.array(self.coords, dtype=np.float64).reshape(-1, 3)

    def __len__(self):
        return len(self.symbols)


def nucRepulsion(nuc: NuclearCluster) -> float:
    """nucRepulsion (src/Particles.jl:197-210)."""
    Z = np.asarray(nuc.charges, dtype=np.float64)
    R = np.asarray(nuc.positions, dtype=np.float64).reshape(-1, 3)
    if len(Z) < 2:
        return 0.0
    i, j = np.triu_indices(len(Z), 1)
    d = np.sqrt(np.sum((R[i] - R[j]) ** 2, axis=1))
    return float(np.sum(Z[i] * Z[j] / d))


@dataclass
class FlatBasis:
    """A basis flattened to the arrays of ``qb_basis``: function f owns primitives
    fun_ptr[f]..fun_ptr[f+1]-1, each with its own centre, Cartesian powers,
    exponent and effective weight (normalisation baked in)."""
    fun_ptr: np.ndarray      # int32 [nfun+1]
    center: np.ndarray       # float64 [nprim, 3]
    ijk: np.ndarray          # int32 [nprim, 3]
    alpha: np.ndarray        # float64 [nprim]
    weight: np.ndarray       # float64 [nprim]

    @property
    def nfun(self):
        return len(self.fun_ptr) - 1


def flatten(basis) -> FlatBasis:
    """Per-primitive arrays of a list of PrimitiveOrb / CompositeOrb (getOrbCorePointers,
    Framework.jl:784-825)."""
    ptr, cen, ijk, alp, w = [0], [], [], [], []
    for orb in basis:
        items = [(orb, orb.weight())] if isinstance(orb, PrimitiveOrb) else orb.effective()
        for p, wt in items:
            cen.append(p.center)
            ijk.append(p.ijk)
            alp.append(p.alpha)
            w.append(wt)
        ptr.append(len(alp))
    return FlatBasis(np.asarray(ptr, np.int32), np.asarray(cen, np.float64).reshape(-1, 3),
                     np.asarray(ijk, np.int32).reshape(-1, 3), np.asarray(alp, np.float64),
                     np.asarray(w, np.float64))


def prepareSpinConfiguration(nuc: NuclearCluster, offset: int = 0):
    """Neutral occupation split (nAlpha >= nBeta) (src/Particles.jl:146-170)."""
    total = int(sum(NUCLEAR_CHARGE[s] for s in nuc.symbols)) + offset
    if total < 0:
        raise ValueError("DomainError: negative electron count")
    nb = total // 2
    return (total - nb, nb)
