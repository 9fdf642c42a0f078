"""The allocation-free J/K entry point (qb_jk_noalloc) against the regular one (qb_jk)
and the exact (quad-precision) oracle.

Callers of qb_jk_noalloc cannot allocate device memory themselves, so this test
allocates the device buffers (with torch) and the entry point must fill them
without allocating: two calls in a row must both reproduce qb_jk's J and K, the
device's free memory must not change across a call, and bad basis data must come
back as status codes.  Collected last so that a failure here never hides the other
tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-11   # same bound as the generic-path J/K test


def _dev(torch, a, dtype):
    return torch.tensor(np.ascontiguousarray(a).reshape(-1), dtype=dtype, device="cuda:0")


def test_jk_noalloc_matches_qb_jk_twice(qb, oracle):
    torch = pytest.importorskip("torch")
    from quiqbox_gb300 import _lib as L
    from quiqbox_gb300.workloads import random_density, random_shell_molecule
    lib = qb.load_library()
    atoms, coords, bs = random_shell_molecule(n_h=2, n_heavy=1, box=4.0, min_dist=1.0, seed=11)
    fb = qb.flatten(bs)
    n = fb.nfun
    D = random_density(n, 11)
    Jr, Kr = qb.jk(fb, D, schwarz=0.0)
    Jx, Kx = oracle.jk(fb, D, exact=True)   # the reference's recursions in quad precision
    fp = _dev(torch, fb.fun_ptr, torch.int32)
    cen = _dev(torch, fb.center, torch.float64)
    ijk = _dev(torch, fb.ijk, torch.int32)
    al = _dev(torch, fb.alpha, torch.float64)
    w = _dev(torch, fb.weight, torch.float64)
    ip = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_int))
    dp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
    basis = L.QBBasis(n, ip(fp), dp(cen), ip(ijk), dp(al), dp(w))
    dD = _dev(torch, D.reshape(-1, order="F"), torch.float64)
    dJ = torch.empty(n * n, dtype=torch.float64, device="cuda:0")
    dK = torch.empty(n * n, dtype=torch.float64, device="cuda:0")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    scale = max(np.abs(Jr).max(), 1.0)
    for call in range(2):
        dJ.fill_(float("nan"))
        dK.fill_(float("nan"))
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = lib.qb_jk_noalloc(C.byref(basis), C.c_void_p(dD.data_ptr()), C.c_void_p(dJ.data_ptr()),
                               C.c_void_p(dK.data_ptr()), stream)
        assert rc == 0
        torch.cuda.synchronize()
        if call == 1:   # after the first call's one-time set-up, a call leaves device memory untouched
            assert torch.cuda.mem_get_info()[0] == free0
        J = dJ.cpu().numpy().reshape((n, n), order="F")
        K = dK.cpu().numpy().reshape((n, n), order="F")
        assert np.abs(J - Jr).max() < TOL * scale
        assert np.abs(K - Kr).max() < TOL * scale
        assert np.abs(J - Jx).max() < 1e-12 * scale
        assert np.abs(K - Kx).max() < 1e-12 * scale
    # bad basis data, caught by the entry point's own checks before the integral kernels:
    # a non-increasing function pointer (QB_ERR_ARG), a non-positive exponent (QB_ERR_DOMAIN),
    # angular momentum above 12 (QB_ERR_UNSUPPORTED)
    fp_bad = fb.fun_ptr.copy()
    fp_bad[2] = fp_bad[1]
    al_bad = fb.alpha.copy()
    al_bad[0] = 0.0
    ijk_bad = fb.ijk.copy()
    ijk_bad[0] = (13, 0, 0)
    for (fpa, ija, ala), code in (((fp_bad, fb.ijk, fb.alpha), 1), ((fb.fun_ptr, fb.ijk, al_bad), 3),
                                  ((fb.fun_ptr, ijk_bad, fb.alpha), 8)):
        t_fp, t_ijk, t_al = _dev(torch, fpa, torch.int32), _dev(torch, ija, torch.int32), _dev(torch, ala, torch.float64)
        bad = L.QBBasis(n, ip(t_fp), dp(cen), ip(t_ijk), dp(t_al), dp(w))
        assert lib.qb_jk_noalloc(C.byref(bad), C.c_void_p(dD.data_ptr()), C.c_void_p(dJ.data_ptr()),
                                 C.c_void_p(dK.data_ptr()), stream) == code
    # beyond the stated maximum (nfun <= 512): rejected before any pointer is touched
    big = L.QBBasis(513, ip(fp), dp(cen), ip(ijk), dp(al), dp(w))
    assert lib.qb_jk_noalloc(C.byref(big), C.c_void_p(dD.data_ptr()), C.c_void_p(dJ.data_ptr()),
                             C.c_void_p(dK.data_ptr()), stream) == 2
