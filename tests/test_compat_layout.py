"""The drop-in shim's restated struct layout equals the reference's (its
own header compiled by oracle/Makefile), and the shim exports the
reference's entry-point names.  CPU only."""
import ctypes

import numpy as np
import pytest

import oracle as O
import refapi


def test_shim_exports_reference_names():
    L = refapi.shim()
    for name in ("pgmres", "ebemv", "Diag_precond", "Diag_precond_EBE_setup", "NO_precond", "NO_precond_setup"):
        assert hasattr(L, name), name


def test_python_mirror_matches_shim_header():
    out = np.zeros(64, dtype=np.int64)
    refapi.shim().fgc_sst_layout(out)
    assert list(out[:37]) == refapi.layout_offsets()


@pytest.mark.skipif(not O.ref_available(), reason="reference build (oracle/_ref) not present")
def test_shim_layout_matches_reference_header():
    ours = np.zeros(64, dtype=np.int64)
    refapi.shim().fgc_sst_layout(ours)
    theirs = O.ref_layout()
    assert np.array_equal(ours[:37], theirs[:37])


@pytest.mark.parametrize("kind,names", [
    ("ns", ("pgmres", "ebemvNDOF3", "BlockDiagDOF3_precond", "BlockDiagDOF3_precond_EBE_setup", "Diag_precond",
            "Diag_precond_EBE_setup", "NO_precond", "NO_precond_setup")),
    ("euler", ("pgmres", "ebemvNDOF4", "BlockDiag_precond", "BlockDiag_precond_EBE_setup", "Diag_precond",
               "Diag_precond_EBE_setup", "NO_precond", "NO_precond_setup"))])
def test_block_shims_export_reference_names(kind, names):
    L = refapi.block_shim(kind)
    for name in names:
        assert hasattr(L, name), name


@pytest.mark.parametrize("kind", ["ns", "euler"])
def test_block_python_mirror_matches_shim_header(kind):
    out = np.zeros(64, dtype=np.int64)
    getattr(refapi.block_shim(kind), refapi._KINDS[kind]["layout"])(out)
    assert list(out[:31]) == refapi.block_layout_offsets(kind)


@pytest.mark.parametrize("kind", ["ns", "euler"])
def test_block_shim_layout_matches_reference_header(kind):
    R = O.ref_ns() if kind == "ns" else O.ref_euler()
    if R is None:
        pytest.skip("reference build (oracle/_ref) not present")
    theirs = np.zeros(64, dtype=np.int64)
    (R.fr_ns_layout if kind == "ns" else R.fr_eu_layout)(theirs)
    ours = np.zeros(64, dtype=np.int64)
    getattr(refapi.block_shim(kind), refapi._KINDS[kind]["layout"])(ours)
    assert np.array_equal(ours[:31], theirs[:31])


def _tt_shim():
    from parallel_fem_codes_gb300 import build as _b
    _b.build()
    L = ctypes.CDLL(_b.COMPAT_TT)
    L.fgc_tt_layout.argtypes = [np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")]
    L.fgc_tt_layout.restype = None
    return L


def test_tt_shim_exports_reference_names():
    """The transient-transport driver's solve path (pgmres, ebemv, Diag, NO)."""
    L = _tt_shim()
    for name in ("pgmres", "ebemv", "Diag_precond", "Diag_precond_EBE_setup", "NO_precond", "NO_precond_setup"):
        assert hasattr(L, name), name


@pytest.mark.skipif(O.ref_tt() is None, reason="reference transient build (oracle/_ref) not present")
def test_tt_shim_layout_matches_reference_header():
    ours = np.zeros(64, dtype=np.int64)
    _tt_shim().fgc_tt_layout(ours)
    assert np.array_equal(ours[:37], O.ref_tt_layout()[:37])
