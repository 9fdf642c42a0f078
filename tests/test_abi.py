"""C-ABI library: it loads, exports every symbol include/quiqbox_gb300.h declares,
and reports errors as status codes.  No compute call needs a GPU here."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"\b(qb_\w+)\s*\(", h.read_text()))
    return names


def test_header_matches_binding_list(qb):
    assert _declared() == set(qb.EXPORTED)


def test_library_exports_every_declared_symbol(qb):
    qb.load_library()
    lib = ctypes.CDLL(str(qb.LIB_PATH))
    for name in _declared():
        assert hasattr(lib, name), name


def test_default_scf_config_matches_reference(qb):
    # SCFconfig() = ((:DD, :ADIIS, :DIIS), (5e-3, 1e-4, 1e-9)), secondaryConvRatio (1000, 1000),
    # oscillateThreshold 5e-6, maxStep 200, DIIS size 15, damping 0.75 (HartreeFock.jl:16-27)
    from quiqbox_gb300 import _lib as L
    lib = qb.load_library()
    cfg = L.QBSCFConfig()
    lib.qb_scf_config_default(ctypes.byref(cfg))
    assert cfg.nmethod == 3 and list(cfg.method)[:3] == [0, 3, 1]
    assert list(cfg.interval)[:3] == [5e-3, 1e-4, 1e-9]
    assert tuple(cfg.secondary_ratio) == (1000.0, 1000.0)
    assert cfg.oscillate_threshold == 5e-6 and cfg.max_step == 200 and cfg.diis_size == 15
    assert cfg.damp_strength == 0.75 and cfg.guess == 2
    # defaultDIISsolver = :LBFGS (HartreeFock.jl:17) for every method
    assert list(cfg.solver) == [0] * 8


def test_scfconfig_solver_keywords(qb):
    # SCFconfig(methods, intervals, Dict(2=>[:solver=>:LCM])) (HartreeFock.jl:645-648, 1480)
    sc = qb.SCFconfig(("ADIIS", "DIIS", "EDIIS", "DD"), (1e-4, 1e-8, 1e-10, 1e-15),
                      {1: [("solver", "LCM")], 3: [("solver", "SPGB")]})
    assert [sc.solver_of(k) for k in range(4)] == ["LCM", "LBFGS", "SPGB", "LBFGS"]
    with pytest.raises(ValueError):
        qb.SCFconfig(("DIIS",), (1e-8,), {1: [("solver", "BFGS")]})
    with pytest.raises(ValueError):
        qb.SCFconfig(("DIIS",), (1e-8,), {2: [("solver", "LCM")]})


def test_null_arguments_are_rejected_without_device(qb):
    lib = qb.load_library()
    assert lib.qb_create(None, 0) == 1          # QB_ERR_ARG
    assert lib.qb_overlaps(None, None, None) == 1


def test_context_creation_reports_status(qb):
    # Without a GPU qb_create fails with a CUDA status and a message; with one it succeeds.
    try:
        ctx = qb.Context(0)
    except Exception as e:   # noqa: BLE001
        assert "qb_create failed" in str(e)
    else:
        ctx.close()
