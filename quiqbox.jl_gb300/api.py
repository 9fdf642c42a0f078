"""Host-side mirror of Quiqbox.jl's exported integral API and its Hartree–Fock
entry point, each calling the GB300 C ABI.

Names, argument meaning and error behaviour follow the reference:
``overlap(s)``, ``elecKinetic(s)``, ``nucAttraction(s)``, ``coreHamiltonian``,
``elecRepulsion(s)`` (src/Integration/Interface.jl:21-365) and
``runHartreeFock`` with ``HFconfig`` / ``SCFconfig`` (src/HartreeFock.jl:659-1046).
Matrices come back as numpy arrays in the reference's index order.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _lib as L
from .basis import (CompositeOrb, FlatBasis, NuclearCluster, PrimitiveOrb, flatten, nucRepulsion,
                    prepareSpinConfiguration, NUCLEAR_CHARGE)

DimensionMismatch = L.DimensionMismatch
DomainError = L.DomainError


def _ctx(ctx):
    return ctx if ctx is not None else L.default_context()


def _flat(basis) -> FlatBasis:
    if isinstance(basis, FlatBasis):
        return basis
    if isinstance(basis, (PrimitiveOrb, CompositeOrb)):
        basis = [basis]
    basis = list(basis)
    if not basis:
        raise ValueError("AssertionError: the basis set must not be empty")
    return flatten(basis)


def _nuclei(nucs, coords=None):
    """(charges, positions) from a NuclearCluster or from symbol / coordinate lists."""
    if isinstance(nucs, NuclearCluster):
        return nucs.charges, nucs.positions
    if coords is None or len(nucs) != len(coords):
        raise ValueError("AssertionError: `nucs` and `coords` should have the same length.")
    Z = np.array([NUCLEAR_CHARGE[s] if isinstance(s, str) else float(s) for s in nucs], np.float64)
    return Z, np.asarray(coords, np.float64).reshape(-1, 3)


def _matrix(fn, fb, ctx, *extra):
    c = _ctx(ctx)
    b = L.BasisArgs(fb)
    out = np.zeros(fb.nfun * fb.nfun)
    c.check(fn(c.h, b.ref(), *extra, L.dptr(out)))
    return out.reshape((fb.nfun, fb.nfun), order="F")


def overlaps(basis, ctx=None):
    """S_ij = <i|j> (Interface.jl:46)."""
    fb = _flat(basis)
    return _matrix(_ctx(ctx).lib.qb_overlaps, fb, ctx)


def overlap(b1, b2, ctx=None):
    """<b1|b2> (Interface.jl:21)."""
    return overlaps([b1, b2], ctx)[0, 1]


def multipoleMoments(center, degrees, basis, ctx=None):
    """M_ij = <i| prod_k (x_k - C_k)^{n_k} |j> (Interface.jl:95)."""
    fb = _flat(basis)
    C3 = np.ascontiguousarray(np.asarray(center, dtype=np.float64).reshape(3))
    n3 = np.ascontiguousarray(np.asarray(degrees, dtype=np.int32).reshape(3))
    return _matrix(_ctx(ctx).lib.qb_multipole_moments, fb, ctx, L.dptr(C3), L.iptr(n3))


def multipoleMoment(center, degrees, b1, b2, ctx=None):
    """<b1| prod_k (x_k - C_k)^{n_k} |b2> (Interface.jl:71)."""
    return multipoleMoments(center, degrees, [b1, b2], ctx)[0, 1]


def elecKinetics(basis, ctx=None):
    """T_ij = <i|-1/2 ∇²|j> (Interface.jl:143)."""
    return _matrix(_ctx(ctx).lib.qb_elec_kinetics, _flat(basis), ctx)


def elecKinetic(b1, b2, ctx=None):
    return elecKinetics([b1, b2], ctx)[0, 1]


def _with_nuclei(fn, basis, nucs, coords, ctx):
    fb = _flat(basis)
    Z, R = _nuclei(nucs, coords)
    Zc = np.ascontiguousarray(Z)
    Rc = np.ascontiguousarray(R.reshape(-1))
    return _matrix(fn, fb, ctx, len(Zc), L.dptr(Zc), L.dptr(Rc))


def nucAttractions(nucs, coords_or_basis, basis=None, ctx=None):
    """V_ij = -Σ_C Z_C <i|1/|r-R_C||j> (Interface.jl:186-256).

    nucAttractions(nucs, coords, basis) or nucAttractions(nuclearCluster, basis)."""
    if isinstance(nucs, NuclearCluster):
        return _with_nuclei(_ctx(ctx).lib.qb_nuc_attractions, coords_or_basis, nucs, None, ctx)
    return _with_nuclei(_ctx(ctx).lib.qb_nuc_attractions, basis, nucs, coords_or_basis, ctx)


def nucAttraction(nucs, coords, b1, b2=None, ctx=None):
    if isinstance(nucs, NuclearCluster):
        return nucAttractions(nucs, [coords, b1], ctx=ctx)[0, 1]
    return nucAttractions(nucs, coords, [b1, b2], ctx=ctx)[0, 1]


def coreHamiltonian(nucs, coords_or_basis, basis=None, ctx=None):
    """H = T + V (Interface.jl:288-312)."""
    if isinstance(nucs, NuclearCluster):
        return _with_nuclei(_ctx(ctx).lib.qb_core_hamiltonian, coords_or_basis, nucs, None, ctx)
    return _with_nuclei(_ctx(ctx).lib.qb_core_hamiltonian, basis, nucs, coords_or_basis, ctx)


def elecRepulsions(basis, ctx=None):
    """Full (ij|kl) tensor, index order [i, j, k, l] (Interface.jl:356-365)."""
    fb = _flat(basis)
    n = fb.nfun
    c = _ctx(ctx)
    b = L.BasisArgs(fb)
    out = np.zeros(n ** 4)
    c.check(c.lib.qb_elec_repulsions(c.h, b.ref(), L.dptr(out)))
    return out.reshape((n, n, n, n), order="F")


def elecRepulsion_list(basis, quartets, ctx=None):
    """(ij|kl) for explicit 0-based quartets."""
    fb = _flat(basis)
    q = np.ascontiguousarray(np.asarray(quartets, np.int32).reshape(-1, 4))
    c = _ctx(ctx)
    b = L.BasisArgs(fb)
    out = np.zeros(len(q))
    c.check(c.lib.qb_elec_repulsion_list(c.h, b.ref(), len(q), L.iptr(q), L.dptr(out)))
    return out


def elecRepulsion(b1, b2, b3, b4, ctx=None):
    """(b1 b2|b3 b4) (Interface.jl:331)."""
    return float(elecRepulsion_list([b1, b2, b3, b4], [(0, 1, 2, 3)], ctx)[0])


def jk(basis, D, schwarz=1e-12, ctx=None):
    """Direct J_ij = Σ (ij|kl) D_kl and K_ij = Σ (ik|jl) D_kl without a stored ERI tensor."""
    fb = _flat(basis)
    n = fb.nfun
    Dm = np.asarray(D, np.float64)
    if Dm.shape != (n, n):
        raise DimensionMismatch(f"density is {Dm.shape}, basis has {n} functions")
    Df = np.ascontiguousarray(Dm.reshape(-1, order="F"))
    J = np.zeros(n * n)
    K = np.zeros(n * n)
    c = _ctx(ctx)
    b = L.BasisArgs(fb)
    c.check(c.lib.qb_jk(c.h, b.ref(), L.dptr(Df), float(schwarz), L.dptr(J), L.dptr(K)))
    return J.reshape((n, n), order="F"), K.reshape((n, n), order="F")


# ---------------------------------------------------------------------------
RCHartreeFock = "RHF"   # restricted closed-shell (HartreeFock.jl:61)
UOHartreeFock = "UHF"   # unrestricted open-shell (HartreeFock.jl:62)
_METHODS = {"DD": 0, "DIIS": 1, "EDIIS": 2, "ADIIS": 3}
_SOLVERS = {"LBFGS": 0, "SPGB": 1, "LCM": 2}   # ConstraintSolvers (HartreeFock.jl:1480)
_GUESSES = {"CoreH": 0, "GWH": 1, "SAD": 2, "Direct": 3}


@dataclass
class SCFconfig:
    """SCF strategy (HartreeFock.jl:659-693): methods with their stopping thresholds
    (the last converges), per-method keywords keyed by the method's 1-based position as
    the reference's ``Dict(2=>[:solver=>:LCM])`` (``solver``: "LBFGS" (default), "SPGB"
    or "LCM", HartreeFock.jl:1480; ``DIISsize``; ``dampStrength``), secondary convergence
    ratios and the oscillation threshold."""
    methods: Sequence[str] = ("DD", "ADIIS", "DIIS")
    intervals: Sequence[float] = (5e-3, 1e-4, 1e-9)
    config: dict = field(default_factory=dict)
    secondaryConvRatio: Sequence[float] = (1000.0, 1000.0)
    oscillateThreshold: float = 5e-6

    def __post_init__(self):
        if len(self.methods) != len(self.intervals) or not self.methods:
            raise ValueError("AssertionError: methods and intervals must have the same non-zero length")
        for m in self.methods:
            if m not in _METHODS:
                raise ValueError(f"unknown SCF method {m}")
        for idx, kws in self.config.items():
            if not 1 <= int(idx) <= len(self.methods):
                raise ValueError(f"method index {idx} out of range")
            for key, val in dict(kws).items():
                if key == "solver" and val not in _SOLVERS:
                    # getproperty(ConstraintSolvers, solver) (HartreeFock.jl:1482-1487) has no such field
                    raise ValueError(f"unknown DIIS solver {val!r} (LBFGS, SPGB or LCM)")

    def solver_of(self, k: int) -> str:
        """The coefficient solver of method k (0-based)."""
        return dict(self.config.get(k + 1, {})).get("solver", "LBFGS")
        if np.ndim(self.secondaryConvRatio) == 0:
            self.secondaryConvRatio = (float(self.secondaryConvRatio),) * 2

    @classmethod
    def default(cls, threshold=1e-9, secondaryConvRatio=(1000.0, 1000.0), oscillateThreshold=5e-6):
        """SCFconfig(; threshold) (HartreeFock.jl:695-701)."""
        return cls(("DD", "ADIIS", "DIIS"), (5e-3, 1e-4, float(threshold)), {}, secondaryConvRatio,
                   oscillateThreshold)


@dataclass
class HFconfig:
    """Hartree–Fock configuration (HartreeFock.jl:874-904)."""
    type: str = RCHartreeFock
    initial: object = "SAD"       # "CoreH" | "GWH" | "SAD" | tuple of coefficient matrices (Direct)
    strategy: SCFconfig = field(default_factory=SCFconfig)
    maxStep: int = 200
    earlyStop: bool = True
    schwarz: float = 1e-14

    def __post_init__(self):
        if self.maxStep < 1:
            raise DomainError("maxStep must be positive")


@dataclass
class HFfinalInfo:
    """Final values of an SCF run (HartreeFock.jl:791-819)."""
    energy: tuple                 # (E_elec, E_nuc)
    coeff: tuple
    density: tuple
    fock: tuple
    occu: tuple                   # per sector: (orbital energies, occupations)
    converged: object
    steps: int
    spin: tuple


def runHartreeFock(nucInfo, basis, config: Optional[HFconfig] = None, spin=None, ctx=None) -> HFfinalInfo:
    """runHartreeFock (HartreeFock.jl:953-1046) on the GPU.

    nucInfo: NuclearCluster; spin: (nAlpha, nBeta) or None for the neutral,
    maximally paired configuration (prepareSpinConfiguration, src/Particles.jl:146-170)."""
    if not isinstance(nucInfo, NuclearCluster):
        raise ValueError("nucInfo must be a NuclearCluster")
    fb = _flat(basis)
    n = fb.nfun
    na, nb = spin if spin is not None else prepareSpinConfiguration(nucInfo)
    if config is None:
        config = HFconfig(type=RCHartreeFock if (na + nb) % 2 == 0 else UOHartreeFock)
    uhf = config.type == UOHartreeFock
    if not uhf and na != nb:
        raise ValueError("AssertionError: Close-shell system must have the same number of spins for both "
                         "spin orientations.")
    nsec = 2 if uhf else 1
    cfg = L.QBSCFConfig()
    c = _ctx(ctx)
    c.lib.qb_scf_config_default(C.byref(cfg))
    cfg.uhf = int(uhf)
    C0 = None
    if isinstance(config.initial, str):
        cfg.guess = _GUESSES[config.initial]
    else:
        mats = list(config.initial)
        if len(mats) != nsec or any(np.asarray(m).shape != (n, n) for m in mats):
            raise DimensionMismatch("The size/sizes of the input initial orbital coefficient matrix/matrices "
                                    f"does not match the basis-set size ({n}).")
        C0 = np.ascontiguousarray(np.concatenate([np.asarray(m, np.float64).reshape(-1, order="F") for m in mats]))
        cfg.guess = 3
        cfg.C0 = L.dptr(C0)
    st = config.strategy
    cfg.nmethod = len(st.methods)
    for k, (m, iv) in enumerate(zip(st.methods, st.intervals)):
        cfg.method[k] = _METHODS[m]
        cfg.interval[k] = float(iv)
        cfg.solver[k] = _SOLVERS[st.solver_of(k)]
    kw = {}
    for d in st.config.values():
        kw.update(dict(d))
    cfg.diis_size = int(kw.get("DIISsize", 15))
    cfg.damp_strength = float(kw.get("dampStrength", 0.75))
    cfg.secondary_ratio[0] = float(st.secondaryConvRatio[0])
    cfg.secondary_ratio[1] = float(st.secondaryConvRatio[1])
    cfg.oscillate_threshold = float(st.oscillateThreshold)
    cfg.max_step = int(config.maxStep)
    cfg.early_stop = int(bool(config.earlyStop))
    cfg.schwarz = float(config.schwarz)
    Cb, Db, Fb = (np.zeros(nsec * n * n) for _ in range(3))
    eps = np.zeros(nsec * n)
    res = L.QBSCFResult()
    res.C, res.D, res.F, res.eps = L.dptr(Cb), L.dptr(Db), L.dptr(Fb), L.dptr(eps)
    Z = np.ascontiguousarray(nucInfo.charges)
    R = np.ascontiguousarray(nucInfo.positions.reshape(-1))
    b = L.BasisArgs(fb)
    c.check(c.lib.qb_run_hartree_fock(c.h, b.ref(), len(Z), L.dptr(Z), L.dptr(R), int(na), int(nb),
                                      C.byref(cfg), C.byref(res)), allow=(L.QB_ERR_NOT_CONVERGED,))
    mats = lambda buf: tuple(buf[k * n * n:(k + 1) * n * n].reshape((n, n), order="F") for k in range(nsec))
    occ = []
    for k in range(nsec):
        e = eps[k * n:(k + 1) * n]
        if uhf:
            nk = (na, nb)[k]
            mark = (True, False) if k == 0 else (False, True)
            occ.append((e, [mark if i < nk else (False, False) for i in range(n)]))
        else:
            occ.append((e, [(True, True) if 2 * (i + 1) <= na + nb else (False, False) for i in range(n)]))
    conv = {0: False, 1: True, 2: True}[res.converged]
    return HFfinalInfo((res.E_elec, nucRepulsion(nucInfo)), mats(Cb), mats(Db), mats(Fb), tuple(occ), conv,
                       res.steps, (na, nb))


def diis_coefficients(B, v=None, c0=None, solver="LBFGS", convex=False, ctx=None):
    """One DIIS coefficient solve on the device (constraintSolver!, HartreeFock.jl:1479-1487):
    minimise v.c/s + c^T B c/(2 s^2), s = sum(c), with c >= 0 when ``convex`` (EDIIS /
    ADIIS).  ``c0`` is the starting point (default 1, 2, ..., m, as a new subspace starts).
    Returns (normalised c, solver iterations)."""
    if solver not in _SOLVERS:
        raise ValueError(f"unknown DIIS solver {solver!r} (LBFGS, SPGB or LCM)")
    Bm = np.asarray(B, np.float64)
    m = Bm.shape[0]
    if Bm.shape != (m, m):
        raise DimensionMismatch("B must be square")
    Bf = np.ascontiguousarray(Bm.reshape(-1, order="F"))
    vv = None if v is None else np.ascontiguousarray(np.asarray(v, np.float64).reshape(m))
    c = np.ascontiguousarray(np.arange(1.0, m + 1) if c0 is None else np.asarray(c0, np.float64).reshape(m)).copy()
    it = C.c_int(0)
    cx = _ctx(ctx)
    cx.check(cx.lib.qb_diis_coefficients(cx.h, _SOLVERS[solver], int(bool(convex)), m, L.dptr(Bf),
                                         None if vv is None else vv.ctypes.data_as(C.c_void_p), L.dptr(c),
                                         C.byref(it)))
    return c, it.value


def jk_autotune(basis, D, schwarz=1e-12, repeats=1, ctx=None):
    """Times every compiled kernel variant of every angular-momentum class of the direct
    J/K build on this basis and density and keeps the fastest per class in the context
    (qb_jk_autotune).  Returns {class "la lb lc ld": variant}."""
    c = _ctx(ctx)
    fb = _flat(basis)
    b = L.BasisArgs(fb)
    Df = np.ascontiguousarray(np.asarray(D, dtype=np.float64).reshape(-1, order="F"))
    c.check(c.lib.qb_jk_prepare(c.h, b.ref(), C.c_double(schwarz)))
    c.check(c.lib.qb_jk_upload_density(c.h, L.dptr(Df)))
    chosen = np.zeros(32, np.int32)
    c.check(c.lib.qb_jk_autotune(c.h, int(repeats), L.iptr(chosen)))
    st = L.QBJKStats()
    c.check(c.lib.qb_jk_get_stats(c.h, C.byref(st)))
    return {"".join(str(v) for v in st.class_l[k]): int(chosen[k]) for k in range(st.nclass)}


def eigh_lowest(A, k, ctx=None):
    """k lowest eigenpairs of the symmetric matrix A on the device (qb_eigh_lowest)."""
    c = _ctx(ctx)
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    Af = np.ascontiguousarray(A.reshape(-1, order="F"))
    w = np.zeros(k)
    Y = np.zeros(n * k)
    c.check(c.lib.qb_eigh_lowest(c.h, n, k, L.dptr(Af), L.dptr(w), L.dptr(Y)))
    return w, Y.reshape((n, k), order="F")


def computeBoysSequence(T, M, path=0, ctx=None):
    """F_0..F_M at every T (array of shape T.shape + (M+1,)), evaluated on the device.

    Mirrors computeBoysSequence (src/Integration/Engines/BoysFunction.jl:67-77).
    path 0 is the evaluator of the ERI class kernels (M <= 8), path 1 that of the
    generic kernels (M <= 32)."""
    c = _ctx(ctx)
    T = np.ascontiguousarray(np.asarray(T, dtype=np.float64))
    flat = T.reshape(-1)
    out = np.empty((flat.size, M + 1))
    c.check(c.lib.qb_boys(c.h, C.c_int(flat.size), L.dptr(flat), C.c_int(M), C.c_int(path), L.dptr(out)))
    return out.reshape(T.shape + (M + 1,))


def computeBoysFunc(T, m, ctx=None):
    """F_m(T) on the device (computeBoysFunc, src/Integration/Engines/BoysFunction.jl:62-64)."""
    return float(computeBoysSequence(np.array([T]), m, path=1 if m > 8 else 0, ctx=ctx)[0, m])


def _torch_float64():
    import torch
    return torch.float64


@dataclass
class BatchSCFConfig:
    """Configuration of runHartreeFockBatched (qb_batch_config)."""
    conv_energy: float = 1e-10
    conv_density: float = 1e-8
    max_iter: int = 200
    diis_size: int = 15
    schwarz: float = 1e-14
    iters_per_graph: int = 4
    eigensolver: int = 0          # 0: tridiagonal occupied-subspace solver; 1: Jacobi
    jacobi_sweeps: int = 0        # Jacobi sweeps per SCF iteration; 0 = to convergence
    fallback_iter: int = 0        # with initial densities: restart from CoreH after this many iterations
    strategy: Optional[SCFconfig] = None   # None: one DIIS method at conv_energy, exact coefficients;
                                           # else the reference's method sequence, e.g. SCFconfig.default(1e-10)
    earlyStop: bool = True
    dampStrength: float = 0.75
    digest_chunk: int = 0         # stored quartets per digest block (0: chosen by timing on the batch)


@dataclass
class BatchSCFResult:
    energies: np.ndarray          # total energies (electronic + nuclear repulsion), Ha
    elec_energies: np.ndarray
    iterations: np.ndarray
    converged: np.ndarray
    jacobi_sweeps: np.ndarray
    nfun: np.ndarray
    ms_integrals: float
    ms_scf: float
    quartets: int
    prim_quartets: int
    eri_doubles: int
    graph_launches: int
    densities: Optional[list] = None   # final per-spin densities (return_densities=True)
    restarted: Optional[np.ndarray] = None   # restarted from the core-Hamiltonian guess (fallback_iter)
    digest_chunk: int = 0                    # digest chunk size chosen by timing on the batch


_TRIU = {}


def _nuc_repulsions(nnuc, Z, R):
    """nucRepulsion (src/Particles.jl:197-210) of every molecule of a batch at once:
    nuclei concatenated (charges Z, positions R, nnuc per molecule)."""
    nnuc = np.asarray(nnuc, np.int64)
    start = np.concatenate([[0], np.cumsum(nnuc)[:-1]])
    ii, jj, mol = [], [], []
    for m, (n, s) in enumerate(zip(nnuc, start)):
        if n < 2:
            continue
        t = _TRIU.get(n)
        if t is None:
            t = _TRIU[n] = np.triu_indices(n, 1)
        ii.append(t[0] + s)
        jj.append(t[1] + s)
        mol.append(np.full(len(t[0]), m))
    out = np.zeros(len(nnuc))
    if ii:
        i, j, mol = np.concatenate(ii), np.concatenate(jj), np.concatenate(mol)
        P = R.reshape(-1, 3)
        d = np.sqrt(np.sum((P[i] - P[j]) ** 2, axis=1))
        out = np.bincount(mol, weights=Z[i] * Z[j] / d, minlength=len(nnuc))
    return out


def runHartreeFockBatched(molecules, config: Optional[BatchSCFConfig] = None, ctx=None,
                          initial_densities=None, return_densities=False) -> BatchSCFResult:
    """Closed-shell HF of many molecules in one call (qb_run_rhf_batched).

    molecules: sequence of (nucInfo, basis) or (nucInfo, basis, charge); nucInfo a
    NuclearCluster, basis a list of orbitals or a FlatBasis.  Each molecule is what
    runHartreeFock (HartreeFock.jl:972-1046) would solve with initial=:CoreH and the
    strategy of ``config`` (default: :DIIS with exact coefficients), all of them sharing
    every launch."""
    c = _ctx(ctx)
    cfg = config or BatchSCFConfig()
    nmol = len(molecules)
    args, nnuc, Zs, Rs, nocc, enn, nf = [], [], [], [], [], [], []
    for mol in molecules:
        nuc, basis = mol[0], mol[1]
        charge = mol[2] if len(mol) > 2 else 0
        fb = _flat(basis)
        Zm = nuc.charges
        nel = int(round(Zm.sum())) - int(charge)
        if nel <= 0 or nel % 2:
            raise DomainError("closed-shell molecule needs a positive even electron count")
        args.append(L.BasisArgs(fb))
        nnuc.append(len(Zm))
        Zs.append(Zm)
        Rs.append(nuc.positions.reshape(-1))
        nocc.append(nel // 2)
        nf.append(fb.nfun)
    bases = (L.QBBasis * nmol)(*[a.s for a in args])
    nnuc_a = np.ascontiguousarray(nnuc, np.int32)
    Z = np.ascontiguousarray(np.concatenate(Zs), np.float64)
    R = np.ascontiguousarray(np.concatenate(Rs), np.float64)
    enn = _nuc_repulsions(nnuc_a, Z, R)
    nocc_a = np.ascontiguousarray(nocc, np.int32)
    d0 = None
    d0_dev = None
    if initial_densities is not None and hasattr(initial_densities, "data_ptr"):
        # one float64 device (or host) tensor: all molecules' column-major densities, concatenated
        if initial_densities.dtype != _torch_float64() or initial_densities.numel() < sum(n * n for n in nf) \
                or not initial_densities.is_contiguous():
            raise DimensionMismatch("initial density tensor: contiguous float64 with sum(nfun^2) entries")
        d0_dev = C.cast(initial_densities.data_ptr(), C.POINTER(C.c_double))
    elif initial_densities is not None:
        if len(initial_densities) != nmol:
            raise DimensionMismatch("one initial density per molecule")
        parts = []
        for D, n in zip(initial_densities, nf):
            D = np.asarray(D, dtype=np.float64)
            if D.shape != (n, n):
                raise DimensionMismatch("initial density shape")
            parts.append(D.reshape(-1, order="F"))
        d0 = np.ascontiguousarray(np.concatenate(parts))
    qcfg = L.QBBatchConfig()
    c.lib.qb_batch_config_default(C.byref(qcfg))
    qcfg.conv_energy, qcfg.conv_density, qcfg.max_iter = cfg.conv_energy, cfg.conv_density, cfg.max_iter
    qcfg.diis_size, qcfg.schwarz, qcfg.iters_per_graph = cfg.diis_size, cfg.schwarz, cfg.iters_per_graph
    qcfg.initial_density = L.dptr(d0) if d0 is not None else d0_dev
    qcfg.eigensolver, qcfg.jacobi_sweeps, qcfg.fallback_iter = cfg.eigensolver, cfg.jacobi_sweeps, cfg.fallback_iter
    qcfg.early_stop, qcfg.damp_strength = int(bool(cfg.earlyStop)), float(cfg.dampStrength)
    qcfg.digest_chunk = int(cfg.digest_chunk)
    if cfg.strategy is not None:
        st = cfg.strategy
        if len(st.methods) > 8:
            raise ValueError("at most 8 SCF methods")
        qcfg.nmethod = len(st.methods)
        for k, (m, iv) in enumerate(zip(st.methods, st.intervals)):
            qcfg.method[k] = _METHODS[m]
            qcfg.interval[k] = float(iv)
            qcfg.solver[k] = _SOLVERS[st.solver_of(k)]
        qcfg.secondary_ratio[0] = float(st.secondaryConvRatio[0])
        qcfg.secondary_ratio[1] = float(st.secondaryConvRatio[1])
        qcfg.oscillate_threshold = float(st.oscillateThreshold)
    E = np.zeros(nmol)
    it = np.zeros(nmol, np.int32)
    conv = np.zeros(nmol, np.int32)
    sw = np.zeros(nmol, np.int32)
    dout = np.zeros(sum(n * n for n in nf)) if return_densities else None
    rst = np.zeros(nmol, np.int32)
    res = L.QBBatchResult(L.dptr(E), L.iptr(it), L.iptr(conv), L.iptr(sw), 0.0, 0.0, 0, 0, 0, 0,
                          L.dptr(dout) if dout is not None else None, L.iptr(rst))
    c.check(c.lib.qb_run_rhf_batched(c.h, nmol, bases, L.iptr(nnuc_a), L.dptr(Z), L.dptr(R), L.iptr(nocc_a),
                                     C.byref(qcfg), C.byref(res)))
    dens = None
    if dout is not None:
        dens, off = [], 0
        for n in nf:
            dens.append(dout[off:off + n * n].reshape((n, n), order="F"))
            off += n * n
    return BatchSCFResult(E + enn, E, it, conv.astype(bool), sw, np.array(nf), res.ms_integrals,
                          res.ms_scf, int(res.quartets), int(res.prim_quartets), int(res.eri_doubles),
                          int(res.graph_launches), dens, rst.astype(bool), int(res.digest_chunk))


def fp64_peak(ctx=None):
    """Measured FP64 FMA throughput of the device (TFLOP/s)."""
    c = _ctx(ctx)
    out = C.c_double()
    c.check(c.lib.qb_fp64_peak(c.h, C.byref(out)))
    return out.value


def fp64_dmma_peak(ctx=None):
    """Measured FP64 tensor-core (mma.sync m8n8k4) throughput of the device (TFLOP/s)."""
    c = _ctx(ctx)
    out = C.c_double()
    c.check(c.lib.qb_fp64_dmma_peak(c.h, C.byref(out)))
    return out.value


def device_info(ctx=None):
    c = _ctx(ctx)
    sm, ma, mi = C.c_int(), C.c_int(), C.c_int()
    c.check(c.lib.qb_device_info(c.h, C.byref(sm), C.byref(ma), C.byref(mi)))
    return {"sm_count": sm.value, "cc": (ma.value, mi.value)}
