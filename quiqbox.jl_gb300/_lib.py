"""ctypes binding of ``libquiqbox_gb300.so`` (the C ABI of include/quiqbox_gb300.h).

The product path has no CPU fallback: if the CUDA library is not built or the
device cannot run it, every call raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libquiqbox_gb300.so"

QB_OK, QB_ERR_ARG, QB_ERR_DIM, QB_ERR_DOMAIN, QB_ERR_CUDA, QB_ERR_TIMEOUT, QB_ERR_NOT_CONVERGED, \
    QB_ERR_NOMEM, QB_ERR_UNSUPPORTED = range(9)

# Symbols declared by include/quiqbox_gb300.h
EXPORTED = ["qb_create", "qb_destroy", "qb_last_error", "qb_device_info", "qb_overlaps", "qb_elec_kinetics",
            "qb_nuc_attractions", "qb_core_hamiltonian", "qb_elec_repulsions", "qb_elec_repulsion_list", "qb_jk",
            "qb_jk_prepare", "qb_jk_upload_density", "qb_jk_execute", "qb_jk_download", "qb_jk_get_stats", "qb_jk_pair_table",
            "qb_scf_config_default", "qb_run_hartree_fock", "qb_fp64_peak", "qb_jk_noalloc", "qb_boys", "qb_multipole_moments",
            "qb_batch_config_default", "qb_run_rhf_batched", "qb_jk_autotune",
            "qb_bf16_gemm_nt", "qb_gelu_forward", "qb_gelu_backward", "qb_f32_to_bf16", "qb_bf16_transpose",
            "qb_colsum", "qb_mse_grad", "qb_adam_step", "qb_adjoint_jk", "qb_eigh_lowest",
            "qb_guess_features", "qb_guess_assemble", "qb_diis_coefficients", "qb_jk_quartet_list", "qb_jk_class_times", "qb_fp64_dmma_peak"]


class DimensionMismatch(ValueError):
    """Sizes do not agree (Julia's DimensionMismatch)."""


class DomainError(ValueError):
    """Argument outside its domain (Julia's DomainError)."""


class QBError(RuntimeError):
    pass


class QBBasis(C.Structure):
    _fields_ = [("nfun", C.c_int), ("fun_ptr", C.POINTER(C.c_int)), ("center", C.POINTER(C.c_double)),
                ("ijk", C.POINTER(C.c_int)), ("alpha", C.POINTER(C.c_double)), ("weight", C.POINTER(C.c_double))]


class QBJKStats(C.Structure):
    _fields_ = [("shell_path", C.c_int), ("nshell", C.c_int), ("npair", C.c_int), ("nclass", C.c_int),
                ("quartets", C.c_int64), ("prim_quartets", C.c_int64), ("flops", C.c_double),
                ("ms_last", C.c_double), ("class_quartets", C.c_int64 * 32),
                ("class_prim_quartets", C.c_int64 * 32), ("class_l", (C.c_int * 4) * 32)]


class QBSCFConfig(C.Structure):
    _fields_ = [("uhf", C.c_int), ("guess", C.c_int), ("C0", C.POINTER(C.c_double)), ("nmethod", C.c_int),
                ("method", C.c_int * 8), ("interval", C.c_double * 8), ("secondary_ratio", C.c_double * 2),
                ("oscillate_threshold", C.c_double), ("max_step", C.c_int), ("early_stop", C.c_int),
                ("diis_size", C.c_int), ("damp_strength", C.c_double), ("schwarz", C.c_double),
                ("solver", C.c_int * 8)]


class QBSCFResult(C.Structure):
    _fields_ = [("E_elec", C.c_double), ("E_nuc", C.c_double), ("converged", C.c_int), ("steps", C.c_int),
                ("dE", C.c_double), ("rms_dD", C.c_double), ("rms_FDS", C.c_double),
                ("C", C.POINTER(C.c_double)), ("D", C.POINTER(C.c_double)), ("F", C.POINTER(C.c_double)),
                ("eps", C.POINTER(C.c_double))]


_lib = None
_lock = threading.Lock()


def load():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                              "(the GPU path has no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        vp = C.c_void_p
        pb = C.POINTER(QBBasis)
        pd = C.POINTER(C.c_double)
        L.qb_create.argtypes = [C.POINTER(vp), C.c_int]
        L.qb_destroy.argtypes = [vp]
        L.qb_destroy.restype = None
        L.qb_last_error.argtypes = [vp]
        L.qb_last_error.restype = C.c_char_p
        L.qb_device_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.qb_overlaps.argtypes = [vp, pb, pd]
        L.qb_elec_kinetics.argtypes = [vp, pb, pd]
        L.qb_nuc_attractions.argtypes = [vp, pb, C.c_int, pd, pd, pd]
        L.qb_core_hamiltonian.argtypes = [vp, pb, C.c_int, pd, pd, pd]
        L.qb_elec_repulsions.argtypes = [vp, pb, pd]
        L.qb_elec_repulsion_list.argtypes = [vp, pb, C.c_int64, C.POINTER(C.c_int), pd]
        L.qb_jk.argtypes = [vp, pb, pd, C.c_double, pd, pd]
        L.qb_jk_prepare.argtypes = [vp, pb, C.c_double]
        L.qb_jk_upload_density.argtypes = [vp, pd]
        L.qb_jk_execute.argtypes = [vp]
        L.qb_jk_download.argtypes = [vp, pd, pd]
        L.qb_jk_get_stats.argtypes = [vp, C.POINTER(QBJKStats)]
        pi = C.POINTER(C.c_int)
        L.qb_jk_pair_table.argtypes = [vp, pi, pi, pi, pi, pi, pd]
        L.qb_jk_quartet_list.argtypes = [vp, C.c_int64, pi, pd, pd]
        L.qb_scf_config_default.argtypes = [C.POINTER(QBSCFConfig)]
        L.qb_scf_config_default.restype = None
        L.qb_run_hartree_fock.argtypes = [vp, pb, C.c_int, pd, pd, C.c_int, C.c_int, C.POINTER(QBSCFConfig),
                                          C.POINTER(QBSCFResult)]
        L.qb_fp64_peak.argtypes = [vp, pd]
        L.qb_diis_coefficients.argtypes = [vp, C.c_int, C.c_int, C.c_int, pd, vp, pd, C.POINTER(C.c_int)]
        L.qb_jk_noalloc.argtypes = [pb, vp, vp, vp, vp]
        for name in EXPORTED:
            f = getattr(L, name)
            if name not in ("qb_destroy", "qb_last_error", "qb_scf_config_default", "qb_batch_config_default"):
                f.restype = C.c_int
        _lib = L
        return L


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Context:
    """One device context (qb_create / qb_destroy)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.qb_create(C.byref(self.h), int(device))
        if rc != QB_OK:
            msg = self.lib.qb_last_error(self.h).decode() if self.h else ""
            if self.h:
                self.lib.qb_destroy(self.h)
            self.h = None
            raise QBError(f"qb_create failed ({rc}): {msg}")

    def close(self):
        if self.h:
            self.lib.qb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc: int, allow=()):
        if rc == QB_OK or rc in allow:
            return rc
        msg = self.lib.qb_last_error(self.h).decode()
        if rc == QB_ERR_DIM:
            raise DimensionMismatch(msg)
        if rc == QB_ERR_DOMAIN:
            raise DomainError(msg)
        if rc == QB_ERR_ARG:
            raise ValueError(msg)
        if rc == QB_ERR_UNSUPPORTED:
            raise NotImplementedError(msg)
        raise QBError(f"status {rc}: {msg}")


class QBBatchConfig(C.Structure):
    _fields_ = [("conv_energy", C.c_double), ("conv_density", C.c_double), ("max_iter", C.c_int),
                ("diis_size", C.c_int), ("schwarz", C.c_double), ("iters_per_graph", C.c_int),
                ("initial_density", C.POINTER(C.c_double)), ("eigensolver", C.c_int), ("jacobi_sweeps", C.c_int),
                ("fallback_iter", C.c_int), ("nmethod", C.c_int), ("method", C.c_int * 8),
                ("interval", C.c_double * 8), ("solver", C.c_int * 8), ("secondary_ratio", C.c_double * 2),
                ("oscillate_threshold", C.c_double), ("early_stop", C.c_int), ("damp_strength", C.c_double),
                ("digest_chunk", C.c_int)]


class QBBatchResult(C.Structure):
    _fields_ = [("energy", C.POINTER(C.c_double)), ("iterations", C.POINTER(C.c_int)),
                ("converged", C.POINTER(C.c_int)), ("jacobi_sweeps", C.POINTER(C.c_int)),
                ("ms_integrals", C.c_double), ("ms_scf", C.c_double), ("quartets", C.c_int64),
                ("prim_quartets", C.c_int64), ("eri_doubles", C.c_int64), ("graph_launches", C.c_int),
                ("density", C.POINTER(C.c_double)), ("restarted", C.POINTER(C.c_int)), ("digest_chunk", C.c_int)]


class BasisArgs:
    """Keeps the numpy arrays of a FlatBasis alive for the duration of a call."""

    def __init__(self, fb):
        self.fp = np.ascontiguousarray(fb.fun_ptr, np.int32)
        self.cen = np.ascontiguousarray(fb.center, np.float64).reshape(-1)
        self.ijk = np.ascontiguousarray(fb.ijk, np.int32).reshape(-1)
        self.alpha = np.ascontiguousarray(fb.alpha, np.float64)
        self.w = np.ascontiguousarray(fb.weight, np.float64)
        self.nfun = len(self.fp) - 1
        self.s = QBBasis(self.nfun, iptr(self.fp), dptr(self.cen), iptr(self.ijk), dptr(self.alpha), dptr(self.w))

    def ref(self):
        return C.byref(self.s)


_default = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context(0)
    return _default
