"""ORACLE — test infrastructure only.

ctypes wrapper of ``oracle/_build/liboracle.so``, the CPU restatement of
Quiqbox.jl's integral engine and Hartree–Fock driver (see oracle_integrals.cpp
and oracle_scf.cpp for the reference citations).  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may use it, and
only as the checker; the GPU product never imports it.
"""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
_lib = None

_d = C.c_double
_i = C.c_int
_i64 = C.c_int64
_pd = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_pi = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def build():
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.qbo_boys.restype = _d
        L.qbo_boys.argtypes = [_d, _i]
        L.qbo_boys_sequence.argtypes = [_d, _i, _pd]
        for name in ("qbo_prim_overlap", "qbo_prim_kinetic"):
            f = getattr(L, name)
            f.restype = _d
            f.argtypes = [_pd, _d, _pi, _pd, _d, _pi]
        L.qbo_prim_nuclear.restype = _d
        L.qbo_prim_nuclear.argtypes = [_pd, _d, _pi, _pd, _d, _pi, _pd]
        L.qbo_prim_eri.restype = _d
        L.qbo_prim_eri.argtypes = [_pd, _d, _pi] * 4
        basis = [_i, _pi, _pd, _pi, _pd, _pd]
        for sfx in ("", "_q"):
            getattr(L, "qbo_one_body" + sfx).argtypes = [_i] + basis + [_i, C.c_void_p, C.c_void_p, _pd]
            getattr(L, "qbo_eri_tensor" + sfx).argtypes = basis + [_pd]
            getattr(L, "qbo_eri_list" + sfx).argtypes = basis + [_i64, _pi, _pd]
            getattr(L, "qbo_jk_list" + sfx).argtypes = basis + [_i64, _pi, _pd, _pd, _pd, _pd, _i]
            getattr(L, "qbo_multipole" + sfx).argtypes = basis + [_pd, _pi, _pd]
        L.qbo_boys_q.restype = _d
        L.qbo_boys_q.argtypes = [_d, _i]
        L.qbo_num_threads.restype = _i
        L.qbo_hartree_fock.restype = _i
        L.qbo_hartree_fock.argtypes = basis + [_i, _pd, _pd, _i, _i, _i, _i, C.c_void_p, _i, _pi,
                                               _pd, _pi, _d, _d, _d, _i, _i, _pd, _pd, _pd, _pd, _pd]
        L.qbo_diis_solve_iter.restype = _i
        L.qbo_diis_solve_iter.argtypes = [_i, _i, _i, _pd, _pd, _pd]
        L.qbo_eigh.argtypes = [_i, _pd, _pd, _pd]
        _lib = L
    return _lib


def _b(fb):
    return (int(fb.nfun), np.ascontiguousarray(fb.fun_ptr, np.int32),
            np.ascontiguousarray(fb.center, np.float64), np.ascontiguousarray(fb.ijk, np.int32),
            np.ascontiguousarray(fb.alpha, np.float64), np.ascontiguousarray(fb.weight, np.float64))


def _v(x, dt=np.float64):
    return np.ascontiguousarray(np.asarray(x, dt))


def boys(x, n):
    return lib().qbo_boys(float(x), int(n))


def boys_sequence(x, n):
    out = np.zeros(n + 1)
    lib().qbo_boys_sequence(float(x), int(n), out)
    return out


def prim_overlap(A, a, la, B, b, lb):
    return lib().qbo_prim_overlap(_v(A), a, _v(la, np.int32), _v(B), b, _v(lb, np.int32))


def prim_kinetic(A, a, la, B, b, lb):
    return lib().qbo_prim_kinetic(_v(A), a, _v(la, np.int32), _v(B), b, _v(lb, np.int32))


def prim_nuclear(A, a, la, B, b, lb, Cpt):
    return lib().qbo_prim_nuclear(_v(A), a, _v(la, np.int32), _v(B), b, _v(lb, np.int32), _v(Cpt))


def prim_eri(p1, p2, p3, p4):
    args = []
    for (c, a, l) in (p1, p2, p3, p4):
        args += [_v(c), float(a), _v(l, np.int32)]
    return lib().qbo_prim_eri(*args)


def _sfx(exact):
    return "_q" if exact else ""


def boys_exact(x, n):
    """F_n(x) of the same algorithm evaluated in quad precision."""
    return lib().qbo_boys_q(float(x), int(n))


def _one_body(kind, fb, Z=None, R=None, exact=False):
    n = fb.nfun
    f = getattr(lib(), "qbo_one_body" + _sfx(exact))
    out = np.zeros((n, n), order="F")
    buf = np.zeros(n * n)
    if Z is None:
        f(kind, *_b(fb), 0, None, None, buf)
    else:
        Zc, Rc = _v(Z), _v(R).reshape(-1)
        f(kind, *_b(fb), len(Zc), Zc.ctypes.data, Rc.ctypes.data, buf)
    out[:] = buf.reshape((n, n), order="F")
    return out


def overlaps(fb, exact=False):
    return _one_body(0, fb, exact=exact)


def kinetics(fb, exact=False):
    return _one_body(1, fb, exact=exact)


def nuc_attractions(fb, Z, R, exact=False):
    return _one_body(2, fb, Z, R, exact=exact)


def multipoles(fb, center, degrees, exact=False):
    """multipoleMoments(center, degrees, basis) (Interface.jl:95), nfun x nfun."""
    n = fb.nfun
    buf = np.zeros(n * n)
    getattr(lib(), "qbo_multipole" + _sfx(exact))(*_b(fb), _v(center), _v(degrees, np.int32), buf)
    return buf.reshape((n, n), order="F").copy()


def eri_tensor(fb, exact=False):
    """(ij|kl) in the reference's canonical orientation; exact=True evaluates in quad precision."""
    n = fb.nfun
    buf = np.zeros(n ** 4)
    getattr(lib(), "qbo_eri_tensor" + _sfx(exact))(*_b(fb), buf)
    return buf.reshape((n, n, n, n), order="F")


def eri_list(fb, quartets, exact=False):
    q = _v(quartets, np.int32).reshape(-1, 4)
    out = np.zeros(len(q))
    getattr(lib(), "qbo_eri_list" + _sfx(exact))(*_b(fb), len(q), q, out)
    return out


def canonical_quartets(n):
    """Function quartets i>=j, k>=l, ij>=kl with their degeneracy weights."""
    pairs = [(i, j) for i in range(n) for j in range(i + 1)]
    q, g = [], []
    for a, (i, j) in enumerate(pairs):
        for (k, l) in pairs[:a + 1]:
            q.append((i, j, k, l))
            g.append((2.0 if i != j else 1.0) * (2.0 if k != l else 1.0) * (2.0 if (i, j) != (k, l) else 1.0))
    return np.asarray(q, np.int32), np.asarray(g, np.float64)


def jk_list(fb, quartets, weights, D, nthreads=0, exact=False):
    """Accumulated (Jp, Kp) for a weighted quartet list (see qbo_jk_list)."""
    n = fb.nfun
    q = _v(quartets, np.int32).reshape(-1, 4)
    Jp = np.zeros(n * n)
    Kp = np.zeros(n * n)
    Dc = np.ascontiguousarray(np.asarray(D, np.float64).reshape(n, n).T).reshape(-1)  # column-major
    getattr(lib(), "qbo_jk_list" + _sfx(exact))(*_b(fb), len(q), q, _v(weights), Dc, Jp, Kp, int(nthreads))
    return Jp.reshape((n, n), order="F"), Kp.reshape((n, n), order="F")


def jk(fb, D, nthreads=0, exact=False):
    """Direct J_ij = Σ (ij|kl) D_kl and K_ij = Σ (ik|jl) D_kl over the canonical quartets."""
    q, g = canonical_quartets(fb.nfun)
    Jp, Kp = jk_list(fb, q, g, D, nthreads, exact)
    return (Jp + Jp.T) / 4, (Kp + Kp.T) / 8


METHODS = {"DD": 0, "DIIS": 1, "EDIIS": 2, "ADIIS": 3}
SOLVERS = {"LBFGS": 0, "SPGB": 1, "LCM": 2}


def diis_solve(solver, convex, v, B, c0):
    """One DIIS coefficient solve (constraintSolver!, HartreeFock.jl:1479-1487) from the
    starting point c0; returns (normalised c, iterations or status)."""
    c = _v(c0).copy()
    Bf = np.ascontiguousarray(np.asarray(B, np.float64).T)   # column-major
    it = lib().qbo_diis_solve_iter(SOLVERS[solver], int(convex), len(c), _v(v), Bf.reshape(-1), c)
    return c, it
GUESSES = {"CoreH": 0, "GWH": 1, "SAD": 2, "Direct": 3}


def hartree_fock(fb, Z, R, nalpha, nbeta, uhf=False, guess="CoreH", C0=None,
                 methods=("DD", "ADIIS", "DIIS"), intervals=(5e-3, 1e-4, 1e-9),
                 secondary=(1000.0, 1000.0), osc=5e-6, max_step=200, early_stop=True, solvers=None):
    n = fb.nfun
    ns = 2 if uhf else 1
    Cout, Dout, Fout = (np.zeros(ns * n * n) for _ in range(3))
    eps = np.zeros(ns * n)
    info = np.zeros(3)
    c0 = None
    if guess == "Direct":
        c0 = np.ascontiguousarray(np.concatenate([np.asarray(c, np.float64).reshape(n, n).T.reshape(-1)
                                                  for c in C0]))
    Zc, Rc = _v(Z), _v(R).reshape(-1)
    st = lib().qbo_hartree_fock(*_b(fb), len(Zc), Zc, Rc, int(nalpha), int(nbeta), int(uhf),
                                GUESSES[guess], None if c0 is None else c0.ctypes.data,
                                len(methods), _v([METHODS[m] for m in methods], np.int32),
                                _v(intervals), _v([SOLVERS[x] for x in (solvers or ["LBFGS"] * len(methods))], np.int32),
                                float(secondary[0]), float(secondary[1]), float(osc),
                                int(max_step), int(early_stop), Cout, Dout, Fout, eps, info)
    if st != 0:
        raise ValueError("oracle Hartree-Fock rejected its arguments")
    mats = lambda b: [b[k * n * n:(k + 1) * n * n].reshape((n, n), order="F") for k in range(ns)]
    return {"E_elec": info[0], "converged": int(info[1]), "steps": int(info[2]),
            "C": mats(Cout), "D": mats(Dout), "F": mats(Fout),
            "eps": [eps[k * n:(k + 1) * n] for k in range(ns)]}


def num_threads():
    return lib().qbo_num_threads()
