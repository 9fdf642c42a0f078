"""Analytic RHF energy gradient with respect to Gaussian basis parameters, by the
adjoint method (basis-set optimisation).

The reference has no analytic gradient (src/Differentiation/Finite.jl holds finite-
difference weights only).  A basis is a
list of contracted Cartesian shells of unnormalised primitives (genGaussTypeOrb with
its default flags, OrbitalBases.jl:199-247): every component function of a shell shares
the shell's centre R, exponents alpha_k and coefficients c_k; the parameters are R,
alpha_k and c_k per shell.

At a converged RHF solution (total density P = 2 C_occ C_occ^T, energy-weighted density
W = 2 C_occ eps_occ C_occ^T) the energy's derivative with respect to one function mu's
shape is, with dmu the derivative of mu (in the first slot only),
    dE = 2 sum_nu P_mu,nu <dmu|H|nu> - 2 sum_nu W_mu,nu <dmu|nu>
         + sum_{nu lam sig} [2 P_mu,nu P_lam,sig - P_mu,lam P_nu,sig] (dmu nu|lam sig).
Each derivative of a primitive x^i y^j z^k e^{-alpha |r - R|^2} is a combination of
primitives with shifted powers: d/dalpha = -(g[i+2] + g[j+2] + g[k+2]),
d/dR_x = 2 alpha g[i+1] - i g[i-1].  These shifted primitives are appended to the basis
as extra functions g; the one-body terms come from the GPU overlap / core-Hamiltonian
kernels over the augmented basis, the two-electron term from qb_adjoint_jk, which
recomputes every (g nu|lam sig) (the backward pass stores no integral) and contracts it
into J[g] and K[g]:  sum [..](g nu|lam sig) = 2 P_mu . J[g] - P_mu . K[g].
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .basis import CompositeOrb, FlatBasis, PrimitiveOrb, cartesian_components, flatten


@dataclass
class GaussShell:
    """One contracted Cartesian shell of unnormalised primitives (the optimisation
    parameters: center, exponents, coefficients)."""
    center: tuple
    L: int
    exponents: list
    coefficients: list

    def orbitals(self):
        out = []
        for ijk in cartesian_components(self.L):
            prims = tuple(PrimitiveOrb(tuple(float(c) for c in self.center), float(a), ijk) for a in self.exponents)
            out.append(CompositeOrb(prims, tuple(float(c) for c in self.coefficients)))
        return out


def shells_basis(shells):
    bs = []
    for sh in shells:
        bs += sh.orbitals()
    return flatten(bs)


_SHIFTS = (("0", (0, 0, 0)), ("+2x", (2, 0, 0)), ("+2y", (0, 2, 0)), ("+2z", (0, 0, 2)),
           ("+1x", (1, 0, 0)), ("+1y", (0, 1, 0)), ("+1z", (0, 0, 1)),
           ("-1x", (-1, 0, 0)), ("-1y", (0, -1, 0)), ("-1z", (0, 0, -1)))


@dataclass
class GradientResult:
    energy: float                  # total RHF energy (electronic + nuclear repulsion)
    d_exponents: list              # per shell, dE/dalpha_k
    d_coefficients: list           # per shell, dE/dc_k
    d_centers: np.ndarray          # (nshell, 3), dE/dR
    scf_steps: int
    extra_functions: int
    timings: dict = field(default_factory=dict)


def tight_scf(conv=1e-12):
    """CoreH guess, DIIS with the exact (Lagrange-multiplier) coefficients, |dE| <= conv and
    RMS(dD) <= 100 conv: tight enough that the energy is stationary to ~conv^2 (what the
    adjoint formula assumes)."""
    from . import api
    return api.HFconfig(initial="CoreH", strategy=api.SCFconfig(("DIIS",), (conv,), {1: [("solver", "LCM")]},
                                                                secondaryConvRatio=(1e6, 100.0)), maxStep=500)


def rhf_energy(nuc, shells, ctx=None, conv=1e-12):
    from . import api
    r = api.runHartreeFock(nuc, shells_basis(shells), tight_scf(conv), ctx=api._ctx(ctx))
    if not r.converged:
        raise RuntimeError("SCF did not converge")
    return float(r.energy[0] + r.energy[1])


def rhf_energy_gradient(nuc, shells, ctx=None, conv=1e-12, scf=None) -> GradientResult:
    """Energy and its gradient with respect to every shell's centre, exponents and
    coefficients for the closed-shell ground state of `nuc` in the basis `shells`."""
    import time
    from . import api
    c = api._ctx(ctx)
    fb = shells_basis(shells)
    n = fb.nfun
    t0 = time.perf_counter()
    cfg = scf or tight_scf(conv)
    r = api.runHartreeFock(nuc, fb, cfg, ctx=c)
    if not r.converged:
        raise RuntimeError("SCF did not converge; the adjoint gradient needs a stationary point")
    t_scf = time.perf_counter() - t0
    nocc = int(round(nuc.charges.sum())) // 2
    Cm = np.asarray(r.coeff[0])
    eps = np.asarray(r.occu[0][0])
    Co = Cm[:, :nocc]
    P = 2.0 * Co @ Co.T
    W = 2.0 * (Co * eps[:nocc]) @ Co.T
    # extra functions: shifted single primitives of every primitive of every function
    fp, cen, ijk, al, w = fb.fun_ptr, np.asarray(fb.center).reshape(-1, 3), np.asarray(fb.ijk).reshape(-1, 3), \
        np.asarray(fb.alpha), np.asarray(fb.weight)
    ext = []       # (function, primitive, shift label, center, alpha, powers)
    for f in range(n):
        for q in range(fp[f], fp[f + 1]):
            for lab, sh in _SHIFTS:
                pw = ijk[q] + np.array(sh)
                if (pw < 0).any():
                    continue
                ext.append((f, q, lab, cen[q], al[q], tuple(int(v) for v in pw)))
    ng = len(ext)
    a_fp = np.concatenate([fp, fp[-1] + 1 + np.arange(ng)]).astype(np.int32)
    a_cen = np.concatenate([cen, np.array([e[3] for e in ext])])
    a_ijk = np.concatenate([ijk, np.array([e[5] for e in ext])]).astype(np.int32)
    a_al = np.concatenate([al, np.array([e[4] for e in ext])])
    a_w = np.concatenate([w, np.ones(ng)])
    aug = FlatBasis(a_fp, a_cen.reshape(-1), a_ijk.reshape(-1), a_al, a_w)
    t1 = time.perf_counter()
    S = api.overlaps(aug, ctx=c)
    H = api.coreHamiltonian(nuc, aug, ctx=c)
    b = L.BasisArgs(aug)
    Pf = np.ascontiguousarray(P.reshape(-1, order="F"))
    Jx = np.zeros(ng * n)
    Kx = np.zeros(ng * n)
    c.check(c.lib.qb_adjoint_jk(c.h, b.ref(), n, L.dptr(Pf), L.dptr(Jx), L.dptr(Kx)))
    t_adj = time.perf_counter() - t1
    Jx = Jx.reshape(ng, n)
    Kx = Kx.reshape(ng, n)
    A = {}
    for k, (f, q, lab, _, _, _) in enumerate(ext):
        g = n + k
        A[(f, q, lab)] = (2.0 * P[f] @ H[g, :n] - 2.0 * W[f] @ S[g, :n] + 2.0 * P[f] @ Jx[k] - P[f] @ Kx[k])
    # chain rule to the shell parameters
    d_exp, d_coef = [], []
    d_cen = np.zeros((len(shells), 3))
    f0 = 0
    for s_i, sh in enumerate(shells):
        comps = cartesian_components(sh.L)
        ge = np.zeros(len(sh.exponents))
        gc = np.zeros(len(sh.exponents))
        for ci, pw in enumerate(comps):
            f = f0 + ci
            for k in range(len(sh.exponents)):
                q = fp[f] + k
                ck, ak = float(sh.coefficients[k]), float(sh.exponents[k])
                gc[k] += A[(f, q, "0")]
                ge[k] += -ck * (A[(f, q, "+2x")] + A[(f, q, "+2y")] + A[(f, q, "+2z")])
                for ax, nm in enumerate("xyz"):
                    v = 2.0 * ak * A[(f, q, "+1" + nm)]
                    if pw[ax] > 0:
                        v -= pw[ax] * A[(f, q, "-1" + nm)]
                    d_cen[s_i, ax] += ck * v
        d_exp.append(ge)
        d_coef.append(gc)
        f0 += len(comps)
    return GradientResult(float(r.energy[0] + r.energy[1]), d_exp, d_coef, d_cen, int(r.steps), ng,
                          {"scf_s": t_scf, "adjoint_s": t_adj})


def config3_systems(seed=0, nprim=2):
    """Basis-gradient workload: an H4 chain (1.4 bohr spacing) and H2O at the H2O
    benchmark geometry; per atom 2 floating s shells and 1 p shell, each of `nprim`
    primitives with exponents log-uniform in [0.2, 8] and coefficients uniform in
    [0.1, 1] (seeded), centred on the atoms."""
    from .basis import NuclearCluster
    from .workloads import H2O_ATOMS, H2O_BENCH_COORDS
    rng = np.random.default_rng(seed)
    systems = []
    for atoms, coords in ((["H"] * 4, [(1.4 * k, 0.0, 0.0) for k in range(4)]),
                          (list(H2O_ATOMS), [tuple(c) for c in H2O_BENCH_COORDS])):
        nuc = NuclearCluster(atoms, coords)
        shells = []
        for x in nuc.coords:
            for L_ in (0, 0, 1):
                ex = np.sort(np.exp(rng.uniform(np.log(0.2), np.log(8.0), nprim)))[::-1]
                co = rng.uniform(0.1, 1.0, nprim)
                shells.append(GaussShell(tuple(x), L_, [float(v) for v in ex], [float(v) for v in co]))
        systems.append((nuc, shells))
    return systems
