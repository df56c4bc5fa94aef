"""ctypes bindings of the oracle (CPU restatement) and of the reference build.

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libfemoracle.so")
# the same restatement built with the reference's -Ofast -march=native: the
# timed CPU baseline only (never a checker)
ORACLE_FAST_SO = os.path.join(HERE, "_build", "libfemoracle_fast.so")
REF_SO = os.path.join(HERE, "_ref", "libref_sst.so")
# the same driver compiled with the reference's -Ofast -march=native: timing only
REF_FAST_SO = os.path.join(HERE, "_ref", "libref_sst_fast.so")
REF_NS_SO = os.path.join(HERE, "_ref", "libref_ns.so")
REF_EU_SO = os.path.join(HERE, "_ref", "libref_euler.so")
# the reference's drivers compiled unchanged but linked against the
# library's drop-in shims (oracle/Makefile `dropin`): same fr_* entry points
DROPIN_SO = {"sst": os.path.join(HERE, "_ref", "libdropin_sst.so"),
             "ns": os.path.join(HERE, "_ref", "libdropin_ns.so"),
             "euler": os.path.join(HERE, "_ref", "libdropin_euler.so")}
DROPIN_TT_SO = os.path.join(HERE, "_ref", "libdropin_tt.so")
# The reference's source tree (used only to build the checker): the
# PFC_REFERENCE_DIR environment variable, else `reference` beside this
# repository.
REF_SRC = os.environ.get("PFC_REFERENCE_DIR") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))
if not os.path.isdir(REF_SRC) and os.path.isdir(os.path.join(HERE, "_build", "refcopy", "00_CommonFiles")):
    REF_SRC = os.path.join(HERE, "_build", "refcopy")     # a private copy made by `make -C oracle refcopy`
_use_fast = False

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_c_int, _c_dbl = ctypes.c_int, ctypes.c_double


def build(ref: bool | None = None, fast: bool = False) -> None:
    """Compile the restatement, and the reference build when its sources exist.
    fast: also the -Ofast -march=native timing build of the restatement."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if fast:
        subprocess.run(["make", "-s", "-C", HERE, "fast"], check=True)
    if ref is None:
        ref = os.path.isdir(REF_SRC)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "ref_fast", f"REF={REF_SRC}"], check=True)
        tt = os.path.isdir(os.path.join(REF_SRC, "02_Transport_Equation"))
        if tt:
            subprocess.run(["make", "-s", "-C", HERE, "ref_tt", f"REF={REF_SRC}"], check=True)
        lib_dir = os.path.join(os.path.dirname(HERE), "parallel_fem_codes_gb300", "_lib")
        if all(os.path.exists(os.path.join(lib_dir, f"libfemgpu_{k}.so")) for k in ("sst", "ns", "euler")):
            subprocess.run(["make", "-s", "-C", HERE, "dropin", f"REF={REF_SRC}"], check=True)
        if tt and os.path.exists(os.path.join(lib_dir, "libfemgpu_tt.so")):
            subprocess.run(["make", "-s", "-C", HERE, "dropin_tt", f"REF={REF_SRC}"], check=True)


_lib = None
_ref = None


def use_fast_build() -> None:
    """Load the -Ofast -march=native build of the restatement instead of the
    checker build (timed CPU baseline only; call before the first oracle
    call of the process)."""
    global _use_fast
    if _lib is not None:
        raise RuntimeError("oracle library already loaded")
    _use_fast = True


def lib():
    global _lib
    if _lib is None:
        so = ORACLE_FAST_SO if _use_fast else ORACLE_SO
        if not os.path.exists(so):
            build(ref=False, fast=_use_fast)
        L = ctypes.CDLL(so)
        L.or_mesh_structured.argtypes = [_c_int, _c_int, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int, _f64p, _f64p, _i32p]
        L.or_fill_lm.argtypes = [_c_int, _c_int, _i32p, _i32p, _i32p, _c_int, _i32p]
        L.or_fill_lm.restype = None
        L.or_lm_adjacency.argtypes = [_c_int, _i32p, _i32p, _i32p, _c_int, _i32p, _i32p]
        L.or_symrcm.argtypes = [_c_int, _i32p, _i32p, _i32p]
        L.or_symrcm.restype = None
        L.or_permutation_of_lm.argtypes = [_c_int, _i32p, _i32p, _i32p, _c_int, _i32p, _i32p, _i32p]
        L.or_ddot.argtypes = [_c_int, _f64p, _f64p]
        L.or_ddot.restype = _c_dbl
        L.or_ebemv3_perm.argtypes = [_c_int, _i32p, _f64p, _i32p, _i32p, _c_int, _f64p, _f64p]
        L.or_ebemv3_perm.restype = None
        L.or_ebemv.argtypes = [_c_int, _c_int, _i32p, _f64p, _c_int, _f64p, _f64p]
        L.or_ebemv.restype = None
        L.or_diag_setup.argtypes = [_c_int, _c_int, _i32p, _f64p, _c_int, _f64p, _f64p, _f64p]
        L.or_diag_setup.restype = None
        L.or_blockdiag_setup.argtypes = [_c_int, _c_int, _c_int, _i32p, _f64p, _i32p, _c_int, _c_int, _f64p, _f64p, _f64p]
        L.or_blockdiag_setup.restype = None
        L.or_blockdiag_apply.argtypes = [_c_int, _c_int, _i32p, _c_int, _f64p, _f64p, _f64p]
        L.or_blockdiag_apply.restype = None
        L.or_build_k_f_supg.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                        ctypes.c_void_p, _f64p, _f64p, _f64p]
        L.or_build_k_f_supg.restype = None
        L.or_transport_process.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                           ctypes.c_void_p, _c_dbl, _c_dbl, _c_int, _c_int, _c_int,
                                           _f64p, ctypes.POINTER(_c_int)]
        L.or_ebe_diag_solve.argtypes = [_c_int, _c_int, _i32p, _f64p, _c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        _f64p, _f64p, _f64p, _c_int, _c_int, _c_dbl, _f64p]
        L.or_ebe_block_solve.argtypes = [_c_int, _c_int, _c_int, _i32p, _i32p, _f64p, _i32p, _c_int, _c_int,
                                         _f64p, _c_int, _c_int, _c_dbl, _f64p]
        L.or_lue_setup.argtypes = [_c_int, _f64p, _f64p]
        L.or_lue_setup.restype = None
        L.or_lue_apply.argtypes = [_c_int, _i32p, _c_int, _f64p, _f64p]
        L.or_lue_apply.restype = None
        L.or_sgs_fwd.argtypes = [_c_int, _i32p, _c_int, _f64p, _f64p]
        L.or_sgs_fwd.restype = None
        L.or_sgs_bwd.argtypes = [_c_int, _i32p, _c_int, _f64p, _f64p]
        L.or_sgs_bwd.restype = None
        L.or_ebe_elem_solve.argtypes = [_c_int, _c_int, _i32p, _f64p, _c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        _f64p, _c_int, _c_int, _c_dbl, _f64p]
        L.or_build_ns.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                  ctypes.c_void_p, _f64p, _f64p, _f64p]
        L.or_build_ns.restype = None
        L.or_ns_process.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                    ctypes.c_void_p, _c_dbl, _c_dbl, _c_int, _c_int, _c_int,
                                    _f64p, ctypes.POINTER(_c_int), ctypes.POINTER(_c_dbl)]
        L.or_build_euler.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                     ctypes.c_void_p, _f64p, _f64p, _f64p, _f64p]
        L.or_build_euler.restype = None
        L.or_build_euler_mfdd.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                          ctypes.c_void_p, _f64p, _f64p, _f64p, _f64p, ctypes.c_void_p,
                                          _f64p, _f64p, _f64p]
        L.or_build_euler_mfdd.restype = None
        L.or_euler_dab.argtypes = [_c_int, _i32p, _c_int, _f64p, _f64p, _f64p]
        L.or_euler_dab.restype = None
        L.or_euler_predictor2.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                          ctypes.c_void_p, ctypes.c_void_p, _c_dbl, _c_int, _c_int,
                                          _f64p, _f64p, _f64p, _f64p, ctypes.c_void_p]
        L.or_euler_predictor.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                         ctypes.c_void_p, ctypes.c_void_p, _c_dbl, _c_int, _c_int,
                                         _f64p, _f64p, ctypes.c_void_p]
        L.or_build_tt.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int, ctypes.c_void_p,
                                  _c_dbl, _c_dbl, _f64p, _f64p, _f64p, _f64p]
        L.or_build_tt.restype = None
        L.or_tt_predictor.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                      ctypes.c_void_p, _c_dbl, _c_dbl, ctypes.c_void_p, _c_dbl, _c_int, _c_int,
                                      _f64p, _f64p, ctypes.c_void_p]
        L.or_build_tt_mfdd.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int, ctypes.c_void_p,
                                       _c_dbl, _c_dbl, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p]
        L.or_build_tt_mfdd.restype = None
        L.or_tt_dab.argtypes = [_c_int, _i32p, _c_int, _f64p, _f64p, _f64p]
        L.or_tt_dab.restype = None
        L.or_tt_predictor2.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                       ctypes.c_void_p, _c_dbl, _c_dbl, ctypes.c_void_p, _c_dbl, _c_int, _c_int,
                                       _f64p, _f64p, _f64p, _f64p, ctypes.c_void_p]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


_loaded = {}


def dropin_available() -> bool:
    return all(os.path.exists(p) for p in DROPIN_SO.values())


_use_ref_fast = False


def ref_fast_available() -> bool:
    """The -Ofast build of the reference's steady-transport driver
    (`make ref_fast`, made by build() where the reference's sources are)."""
    return os.path.exists(REF_FAST_SO)


def use_ref_fast() -> None:
    """Make ref() load the -Ofast build (timed CPU arm only; call before the
    first ref() call of the process)."""
    global _use_ref_fast
    if _ref is not None:
        raise RuntimeError("reference build already loaded")
    _use_ref_fast = True


def using_ref_fast() -> bool:
    return _use_ref_fast


def ref(path=None):
    """The reference's own C (oracle/_ref), or None where it was not built;
    path: another build of the same harness (the drop-in build)."""
    global _ref
    if _use_ref_fast and path is None:
        path = REF_FAST_SO
    if path is not None:
        if path not in _loaded and os.path.exists(path):
            _loaded[path] = _setup_sst(ctypes.CDLL(path))
        return _loaded.get(path)
    if _ref is None and ref_available():
        _ref = _setup_sst(ctypes.CDLL(REF_SO))
    return _ref


def _setup_sst(R):
    if True:
        R.fr_sst_connectivity.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                          _i32p, _i32p, _i32p, _i32p]
        R.fr_sst_build.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                   _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int, _c_dbl, _f64p, _f64p, _f64p]
        R.fr_sst_build.restype = None
        R.fr_sst_process.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int,
                                     _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int, _c_dbl, _c_dbl, _c_dbl,
                                     _c_int, _c_int, _f64p, ctypes.POINTER(_c_int)]
        R.fr_ebemv.argtypes = [_c_int, _c_int, _i32p, _f64p, _i32p, _i32p, _f64p, _f64p]
        R.fr_ebemv.restype = None
        R.fr_diag_pgmres.argtypes = [_c_int, _c_int, _i32p, _f64p, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p,
                                     _c_int, _c_int, _c_dbl]
        if hasattr(R, "fr_sst_timed_solve"):
            R.fr_sst_timed_solve.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int, _c_dbl,
                                             _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int, _c_dbl, _c_int, _c_int, _c_dbl,
                                             ctypes.POINTER(_c_dbl)]
        R.fr_ebe_prec_apply.argtypes = [_c_int, _c_int, _c_int, _i32p, _f64p, _f64p]
        R.fr_ebe_prec_apply.restype = None
        R.fr_ebe_prec_pgmres.argtypes = [_c_int, _c_int, _c_int, _i32p, _f64p, _i32p, _i32p, _f64p, _f64p,
                                         _c_int, _c_int, _c_dbl]
        R.fr_symrcm.argtypes = [_c_int, _c_int, _i32p, _i32p, _i32p]
        R.fr_symrcm.restype = None
        R.fr_sst_layout.argtypes = [np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")]
        R.fr_sst_layout.restype = None
        R.fr_sst_set_form.argtypes = [_c_int, _c_int, _c_int]
        R.fr_sst_set_form.restype = None
    return R


_ref_ns = None


def ref_ns(path=None):
    """The reference's steady Navier-Stokes driver (oracle/_ref), or None."""
    global _ref_ns
    if path is not None:
        if path not in _loaded and os.path.exists(path):
            _loaded[path] = _setup_ns(ctypes.CDLL(path))
        return _loaded.get(path)
    if _ref_ns is None and os.path.exists(REF_NS_SO):
        _ref_ns = _setup_ns(ctypes.CDLL(REF_NS_SO))
    return _ref_ns


def _setup_ns(R):
    if True:
        mesh = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int]
        R.fr_ns_lm.argtypes = mesh + [_i32p]
        R.fr_ns_lm.restype = None
        R.fr_ns_build.argtypes = mesh + [_c_dbl, _f64p, _c_int, _f64p, _f64p, _f64p]
        R.fr_ns_build.restype = None
        R.fr_ns_blockdiag.argtypes = mesh + [_f64p, _f64p, _f64p]
        R.fr_ns_blockdiag.restype = None
        R.fr_ns_ebemv.argtypes = mesh + [_f64p, _f64p, _f64p]
        R.fr_ns_ebemv.restype = None
        R.fr_ns_process.argtypes = mesh + [_c_dbl, _f64p, _c_int, _c_dbl, _c_dbl, _c_int, _c_int, _c_int,
                                           _f64p, ctypes.POINTER(_c_int)]
        R.fr_ns_set_form.argtypes = [_c_int]
        R.fr_ns_set_form.restype = None
        R.fr_ns_layout.argtypes = [np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")]
        R.fr_ns_layout.restype = None
    return R


_ref_eu = None


def ref_euler(path=None):
    """The reference's Euler driver (oracle/_ref), or None."""
    global _ref_eu
    if path is not None:
        if path not in _loaded and os.path.exists(path):
            _loaded[path] = _setup_eu(ctypes.CDLL(path))
        return _loaded.get(path)
    if _ref_eu is None and os.path.exists(REF_EU_SO):
        _ref_eu = _setup_eu(ctypes.CDLL(REF_EU_SO))
    return _ref_eu


def _setup_eu(R):
    if True:
        mesh = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int]
        R.fr_eu_lm.argtypes = mesh + [_i32p]
        R.fr_eu_lm.restype = None
        R.fr_eu_build.argtypes = mesh + [_f64p, _f64p, _c_int, _f64p, _f64p, _f64p, _f64p]
        R.fr_eu_build.restype = None
        R.fr_eu_set_form.argtypes = [_c_int]
        R.fr_eu_set_form.restype = None
        R.fr_eu_blockdiag.argtypes = mesh + [_f64p, _f64p, _f64p]
        R.fr_eu_blockdiag.restype = None
        R.fr_eu_ebemv.argtypes = mesh + [_f64p, _f64p, _f64p]
        R.fr_eu_ebemv.restype = None
        R.fr_eu_predictor.argtypes = mesh + [_f64p, _f64p, _c_int, _f64p, _f64p, _c_int, _c_int, _c_dbl,
                                             _f64p, ctypes.POINTER(_c_dbl)]
        if hasattr(R, "fr_eu_mfdd_build"):
            R.fr_eu_set_invY.argtypes = [_f64p]
            R.fr_eu_set_invY.restype = None
            R.fr_eu_mfdd_build.argtypes = mesh + [_f64p, _f64p, _c_int, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p,
                                                  _f64p, _f64p, _f64p]
            R.fr_eu_mfdd_build.restype = None
        R.fr_eu_layout.argtypes = [np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")]
        R.fr_eu_layout.restype = None
    return R


# ---------------------------------------------------------------- helpers
class _EulerProblem(ctypes.Structure):
    _fields_ = [("gamma", _c_dbl), ("mach", _c_dbl), ("dimensionless", _c_int), ("tolerance", _c_dbl),
                ("alpha", _c_dbl), ("dt", _c_dbl), ("upresc", ctypes.POINTER(_c_dbl)), ("form", _c_int),
                ("uB", ctypes.c_void_p), ("delta_old", ctypes.c_void_p), ("invY", ctypes.POINTER(_c_dbl)),
                ("shock", _c_int)]


class TimeOpts(ctypes.Structure):
    """or_time_opts: the stop tests of Criteria.c."""
    _fields_ = [("stop_by_norm", _c_int), ("max_corrections", _c_int), ("correction_tol", _c_dbl),
                ("steady_state", _c_int), ("final_time", _c_dbl), ("time_tol", _c_dbl), ("max_steps", _c_int),
                ("scheme", _c_int)]

    def as_array(self):
        return np.array([self.stop_by_norm, self.max_corrections, self.correction_tol, self.steady_state,
                         self.final_time, self.time_tol, self.scheme], dtype=np.float64)


class _TimeStats(ctypes.Structure):
    _fields_ = [("steps", _c_int), ("corrections", _c_int), ("gmres_iterations", _c_int), ("t", _c_dbl)]


def _eu_struct(p):
    up = np.ascontiguousarray(p.upresc, dtype=np.float64)
    iy = np.ascontiguousarray(getattr(p, "invY", np.ones(4)), dtype=np.float64)
    s = _EulerProblem(p.gamma, p.mach, int(p.dimensionless), p.tolerance, p.alpha, p.dt,
                      up.ctypes.data_as(ctypes.POINTER(_c_dbl)), int(getattr(p, "form", 0)), None, None,
                      iy.ctypes.data_as(ctypes.POINTER(_c_dbl)), int(getattr(p, "shock", 0)))
    return s, (up, iy)


def build_euler(prob, u=None, du=None):
    """Build_M_K_F_SUPG at (u, du); returns (A[nel, 144], R[neq+1])."""
    m = prob.mesh
    u = prob.initial_state() if u is None else np.ascontiguousarray(u, dtype=np.float64)
    du = np.zeros(m.neq) if du is None else np.ascontiguousarray(du, dtype=np.float64)
    A = np.empty(m.nel * 144)
    R = np.empty(m.neq + 1)
    s, keep = _eu_struct(prob)
    lib().or_build_euler(*_mesh_args(m), ctypes.byref(s), u, du, A, R)
    return A.reshape(m.nel, 144), R


def euler_predictor(prob, topts: TimeOpts, tol=1e-10, kmax=25, lmax=1000, u0=None):
    """Predictor_Old loop; returns (u[neq], a[neq], stats dict)."""
    m = prob.mesh
    u = np.zeros(m.neq + 1)
    u[:m.neq] = prob.initial_state() if u0 is None else u0
    a = np.zeros(m.neq + 1)
    st = _TimeStats()
    s, keep = _eu_struct(prob)
    lib().or_euler_predictor(*_mesh_args(m), ctypes.byref(s), ctypes.byref(topts), tol, kmax, lmax, u, a,
                             ctypes.byref(st))
    return u[:m.neq].copy(), a[:m.neq].copy(), {k: getattr(st, k) for k, _ in st._fields_}


def build_euler_mfdd(prob, u=None, du=None, uB=None, duB=None, dnmv=None):
    """Build_M_F_DD_Transiente ("Predictor2", DD, YZBeta) at (u, du) and the
    bubble unknowns (uB, duB: 4 per element); returns (A[nel, 144],
    F[neq+1], cond[nel, 53] = invN2, R2[4], M2[4][12]).  dnmv (nel, updated
    in place) is Delta_YZBetaNMV's state, None = fresh zeros."""
    m = prob.mesh
    f = lambda a, n: np.zeros(n) if a is None else np.ascontiguousarray(a, dtype=np.float64)
    u = prob.initial_state() if u is None else np.ascontiguousarray(u, dtype=np.float64)
    du, uB, duB = f(du, m.neq), f(uB, 4 * m.nel), f(duB, 4 * m.nel)
    A = np.empty(m.nel * 144)
    F = np.empty(m.neq + 1)
    cond = np.empty(m.nel * 53)
    s, keep = _eu_struct(prob)
    lib().or_build_euler_mfdd(*_mesh_args(m), ctypes.byref(s), u, du, uB, duB,
                              None if dnmv is None else dnmv.ctypes.data, A, F, cond)
    return A.reshape(m.nel, 144), F, cond.reshape(m.nel, 53)


def euler_dab(lm, cond, Da):
    """calculate_DaB of the Euler driver: DaB (4 per element) from Da (neq + 1)."""
    nel = lm.shape[0]
    Da = np.array(Da, dtype=np.float64, copy=True)
    DaB = np.empty(4 * nel)
    lib().or_euler_dab(nel, np.ascontiguousarray(lm, dtype=np.int32).reshape(-1), Da.shape[0] - 1,
                       np.ascontiguousarray(cond, dtype=np.float64).reshape(-1), Da, DaB)
    return DaB


def euler_predictor2(prob, topts: TimeOpts, tol=1e-10, kmax=25, lmax=1000, u0=None):
    """Predictor_New with Build_M_F_DD_Transiente; returns (u, a, uB, aB, stats)."""
    m = prob.mesh
    u = np.zeros(m.neq + 1)
    u[:m.neq] = prob.initial_state() if u0 is None else u0
    a = np.zeros(m.neq + 1)
    uB = np.zeros(4 * max(m.nel, 1))
    aB = np.zeros(4 * max(m.nel, 1))
    st = _TimeStats()
    s, keep = _eu_struct(prob)
    lib().or_euler_predictor2(*_mesh_args(m), ctypes.byref(s), ctypes.byref(topts), tol, kmax, lmax, u, a, uB, aB,
                              ctypes.byref(st))
    return (u[:m.neq].copy(), a[:m.neq].copy(), uB[:4 * m.nel].copy(), aB[:4 * m.nel].copy(),
            {k: getattr(st, k) for k, _ in st._fields_})


def ref_euler_mfdd_build(prob, u, du, uB, duB, Da):
    """The reference's Build_M_F_DD_Transiente (fresh delta states) and its
    calculate_DaB on Da; returns (A[nel, 144], F[neq+1], cond[nel, 53],
    DaB[4 nel])."""
    m = prob.mesh
    R = ref_euler()
    R.fr_eu_set_form(2)
    R.fr_eu_set_invY(np.ascontiguousarray(getattr(prob, "invY", np.ones(4)), dtype=np.float64))
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    A = np.empty(m.nel * 144)
    F = np.zeros(m.neq + 1)
    cond = np.empty(m.nel * 53)
    DaB = np.empty(4 * m.nel)
    R.fr_eu_mfdd_build(*_mesh_args(m), prob.params(), np.ascontiguousarray(prob.coef.reshape(-1)), int(prob.wall),
                       f(u), f(du), f(uB), f(duB), f(Da), A, F, cond, DaB)
    return A.reshape(m.nel, 144), F, cond.reshape(m.nel, 53), DaB


def ref_euler_lm(mesh):
    lm = np.empty(mesh.nel * 12, dtype=np.int32)
    ref_euler().fr_eu_lm(*_mesh_args(mesh), lm)
    return lm.reshape(mesh.nel, 12)


def _ref_eu_form(R, prob):
    """The harness's form code: 0 SUPG + CAU, 1 DD + CAUDD, 3 SUPG + YZBeta,
    4 DD + YZBeta (invY from the problem)."""
    form = int(getattr(prob, "form", 0))
    if int(getattr(prob, "shock", 0)) == 3:
        R.fr_eu_set_invY(np.ascontiguousarray(getattr(prob, "invY", np.ones(4)), dtype=np.float64))
        form += 3
    R.fr_eu_set_form(form)


def ref_euler_build(prob, u=None, du=None):
    m = prob.mesh
    u = prob.initial_state() if u is None else np.ascontiguousarray(u, dtype=np.float64)
    du = np.zeros(m.neq) if du is None else np.ascontiguousarray(du, dtype=np.float64)
    A = np.empty(m.nel * 144)
    R = np.empty(m.neq + 1)
    _ref_eu_form(ref_euler(), prob)
    ref_euler().fr_eu_build(*_mesh_args(m), prob.params(), np.ascontiguousarray(prob.coef.reshape(-1)),
                            int(prob.wall), u, du, A, R)
    return A.reshape(m.nel, 144), R


def ref_euler_blockdiag(mesh, A, F):
    F = np.array(F, dtype=np.float64, copy=True)
    inv = np.empty(mesh.nnodes * 16)
    ref_euler().fr_eu_blockdiag(*_mesh_args(mesh), np.ascontiguousarray(A, dtype=np.float64).reshape(-1), F, inv)
    return inv, F


def ref_euler_ebemv(mesh, A, P):
    Q = np.zeros(mesh.neq + 1)
    ref_euler().fr_eu_ebemv(*_mesh_args(mesh), np.ascontiguousarray(A, dtype=np.float64).reshape(-1),
                            np.ascontiguousarray(P, dtype=np.float64), Q)
    return Q


def ref_euler_predictor(prob, topts: TimeOpts, tol=1e-10, kmax=25, lmax=1000, dropin=False):
    """The reference's Predictor_Old; returns (u[neq], GMRES iterations, final t)."""
    m = prob.mesh
    u = np.zeros(m.neq + 1)
    t = _c_dbl(0.0)
    R = ref_euler(DROPIN_SO["euler"]) if dropin else ref_euler()
    if topts.scheme in (3, 4) or getattr(prob, "form", 0) == 2:
        # "Predictor2" (Predictor_New, _BDF, or _TRBDF2 with form 2): DD + YZBeta, Build_M_F_DD_Transiente
        R.fr_eu_set_form(2)
        R.fr_eu_set_invY(np.ascontiguousarray(getattr(prob, "invY", np.ones(4)), dtype=np.float64))
    else:
        _ref_eu_form(R, prob)
    its = R.fr_eu_predictor(*_mesh_args(m), prob.params(), np.ascontiguousarray(prob.coef.reshape(-1)),
                                      int(prob.wall), np.ascontiguousarray(prob.init), topts.as_array(),
                                      kmax, lmax, tol, u, ctypes.byref(t))
    return u[:m.neq].copy(), its, t.value


class _NSProblem(ctypes.Structure):
    _fields_ = [("reynolds", _c_dbl), ("upresc", ctypes.POINTER(_c_dbl)),
                ("f1", ctypes.POINTER(_c_dbl)), ("f2", ctypes.POINTER(_c_dbl)), ("form", _c_int)]


def _ns_struct(p, form=0):
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (p.upresc, p.f1, p.f2)]
    P = ctypes.POINTER(_c_dbl)
    s = _NSProblem(p.reynolds, keep[0].ctypes.data_as(P), keep[1].ctypes.data_as(P), keep[2].ctypes.data_as(P),
                   form)
    return s, keep


def build_ns(prob, u=None, form=0):
    """Build_K_F_SUPG_PSPG (form 0) or Build_K_F_VMS_DCDD (form 1) at the
    free-dof state u; returns (A[nel, 81], F[neq+1])."""
    m = prob.mesh
    u = np.zeros(m.neq) if u is None else np.ascontiguousarray(u, dtype=np.float64)
    A = np.empty(m.nel * 81)
    F = np.empty(m.neq + 1)
    s, keep = _ns_struct(prob, form)
    lib().or_build_ns(*_mesh_args(m), ctypes.byref(s), u, A, F)
    return A.reshape(m.nel, 81), F


def ns_process(prob, solver_tol=1e-10, nonlinear_tol=1e-3, kmax=30, lmax=1000, max_nonlinear=100, form=0):
    """Picard loop; returns (u[neq], nonlinear its, GMRES its, last ||s||/||u||)."""
    m = prob.mesh
    u = np.zeros(m.neq + 1)
    its, last = _c_int(0), _c_dbl(0.0)
    s, keep = _ns_struct(prob, form)
    nl = lib().or_ns_process(*_mesh_args(m), ctypes.byref(s), solver_tol, nonlinear_tol, kmax, lmax,
                             max_nonlinear, u, ctypes.byref(its), ctypes.byref(last))
    return u[:m.neq].copy(), nl, its.value, last.value


def ref_ns_lm(mesh):
    lm = np.empty(mesh.nel * 9, dtype=np.int32)
    ref_ns().fr_ns_lm(*_mesh_args(mesh), lm)
    return lm.reshape(mesh.nel, 9)


def ref_ns_build(prob, u=None, form=0):
    m = prob.mesh
    ref_ns().fr_ns_set_form(form)
    u = np.zeros(m.neq) if u is None else np.ascontiguousarray(u, dtype=np.float64)
    A = np.empty(m.nel * 81)
    F = np.empty(m.neq + 1)
    ref_ns().fr_ns_build(*_mesh_args(m), prob.reynolds, np.ascontiguousarray(prob.coef.reshape(-1)),
                         int(prob.lid), u, A, F)
    return A.reshape(m.nel, 81), F


def ref_ns_blockdiag(mesh, A, F):
    F = np.array(F, dtype=np.float64, copy=True)
    inv = np.empty(mesh.nnodes * 9)
    ref_ns().fr_ns_blockdiag(*_mesh_args(mesh), np.ascontiguousarray(A, dtype=np.float64).reshape(-1), F, inv)
    return inv, F


def ref_ns_ebemv(mesh, A, P):
    Q = np.zeros(mesh.neq + 1)
    ref_ns().fr_ns_ebemv(*_mesh_args(mesh), np.ascontiguousarray(A, dtype=np.float64).reshape(-1),
                         np.ascontiguousarray(P, dtype=np.float64), Q)
    return Q


def ref_ns_process(prob, solver_tol=1e-10, nonlinear_tol=1e-3, kmax=30, lmax=1000, max_nonlinear=100, form=0,
                   dropin=False):
    m = prob.mesh
    R = ref_ns(DROPIN_SO["ns"]) if dropin else ref_ns()
    R.fr_ns_set_form(form)
    u = np.zeros(m.neq + 1)
    its = _c_int(0)
    R.fr_ns_process(*_mesh_args(m), prob.reynolds, np.ascontiguousarray(prob.coef.reshape(-1)),
                           int(prob.lid), solver_tol, nonlinear_tol, kmax, lmax, max_nonlinear, u,
                           ctypes.byref(its))
    return u[:m.neq].copy(), its.value


class _Problem(ctypes.Structure):
    _fields_ = [("k", _c_dbl), ("gamma", _c_dbl), ("beta", _c_dbl * 2), ("f", _c_dbl),
                ("upresc", ctypes.POINTER(_c_dbl)), ("cau", _c_int), ("form", _c_int), ("h_shock", _c_int),
                ("Re_old", ctypes.c_void_p), ("delta_old", ctypes.c_void_p)]


def _mesh_args(m):
    return (m.nnodes, m.nel, np.ascontiguousarray(m.x), np.ascontiguousarray(m.y),
            np.ascontiguousarray(m.type, dtype=np.int32), np.ascontiguousarray(m.invp, dtype=np.int32),
            np.ascontiguousarray(m.ien, dtype=np.int32).reshape(-1), m.neq)


def _problem_struct(p):
    up = np.ascontiguousarray(p.upresc, dtype=np.float64)
    s = _Problem(p.k, p.gamma, (_c_dbl * 2)(*p.beta), p.f,
                 up.ctypes.data_as(ctypes.POINTER(_c_dbl)), int(p.cau), int(getattr(p, "form", 0)),
                 int(getattr(p, "h_shock", 0)), None, None)
    return s, up


def fill_lm(mesh) -> np.ndarray:
    S = 3 * mesh.ndof
    lm = np.empty(mesh.nel * S, dtype=np.int32)
    lib().or_fill_lm(mesh.nel, mesh.ndof, np.ascontiguousarray(mesh.ien, dtype=np.int32).reshape(-1),
                     mesh.type, mesh.invp, mesh.neq, lm)
    return lm.reshape(mesh.nel, S)


def permutation_of_lm(mesh):
    """(Perm, invPerm, bandwidth[2]) of the local RCM (Permutation_of_LM.c)."""
    n = mesh.neq
    perm = np.empty(n + 1, dtype=np.int32)
    inv = np.empty(n + 1, dtype=np.int32)
    band = np.zeros(2, dtype=np.int32)
    lib().or_permutation_of_lm(mesh.nel, np.ascontiguousarray(mesh.ien, dtype=np.int32).reshape(-1),
                               mesh.type, mesh.invp, n, perm, inv, band)
    return perm, inv, band


def adjacency(mesh):
    n = mesh.neq
    IA = np.empty(n + 1, dtype=np.int32)
    JA = np.empty(mesh.nel * 9 + 1, dtype=np.int32)
    nnz = lib().or_lm_adjacency(mesh.nel, np.ascontiguousarray(mesh.ien, dtype=np.int32).reshape(-1),
                                mesh.type, mesh.invp, n, IA, JA)
    return IA, JA[:nnz].copy()


def symrcm(IA, JA) -> np.ndarray:
    n = IA.shape[0] - 1
    p = np.empty(max(n, 1), dtype=np.int32)
    lib().or_symrcm(n, np.ascontiguousarray(IA, dtype=np.int32), np.ascontiguousarray(JA, dtype=np.int32), p)
    return p[:n]


def build_k_f_supg(prob, u=None):
    m = prob.mesh
    if u is None:
        u = np.zeros(m.neq, dtype=np.float64)
    A = np.empty(m.nel * 9, dtype=np.float64)
    F = np.empty(m.neq + 1, dtype=np.float64)
    s, keep = _problem_struct(prob)
    lib().or_build_k_f_supg(*_mesh_args(m), ctypes.byref(s), np.ascontiguousarray(u, dtype=np.float64), A, F)
    F[m.neq] = 0.0
    return A.reshape(m.nel, 9), F


REF_TT_SO = os.path.join(HERE, "_ref", "libref_tt.so")
_ref_tt = None


_dropin_tt = None


def dropin_tt_available() -> bool:
    return os.path.exists(DROPIN_TT_SO) and os.path.exists(REF_TT_SO)


def ref_tt(dropin=False):
    """The reference's own transient-transport build (oracle/_ref, compiled
    from a private copy of its sources by `make -C oracle ref_tt`), or None;
    dropin=True: the same driver files linked against the library's shim
    (`make -C oracle dropin_tt`)."""
    global _ref_tt, _dropin_tt
    if dropin:
        if _dropin_tt is None and os.path.exists(DROPIN_TT_SO):
            _dropin_tt = _setup_tt(ctypes.CDLL(DROPIN_TT_SO))
        return _dropin_tt
    if _ref_tt is None and os.path.exists(REF_TT_SO):
        _ref_tt = _setup_tt(ctypes.CDLL(REF_TT_SO))
    return _ref_tt


def _setup_tt(R):
    if True:
        R.fr_tt_set_form.argtypes = [_c_int, _c_int, _c_int]
        R.fr_tt_set_form.restype = None
        R.fr_tt_build.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int, _c_dbl, _c_dbl,
                                  _c_dbl, _c_dbl, _c_dbl, _c_int, _c_dbl, _c_dbl, _c_dbl, _f64p, _f64p, _c_int,
                                  _f64p, _f64p]
        R.fr_tt_mfdd_build.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int, _c_dbl, _c_dbl,
                                       _c_dbl, _c_dbl, _c_dbl, _c_int, _c_dbl, _c_dbl, _c_dbl, _f64p, _f64p,
                                       _f64p, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p]
        R.fr_tt_predictor2.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int, _c_dbl, _c_dbl,
                                       _c_dbl, _c_dbl, _c_dbl, _c_int, _c_dbl, _c_dbl, _c_dbl, _i32p, _i32p,
                                       _f64p, _f64p, _c_int, _c_int, _c_dbl, _f64p]
        R.fr_tt_predictor1.argtypes = R.fr_tt_predictor2.argtypes
        R.fr_tt_layout.argtypes = [np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")]
        R.fr_tt_layout.restype = None
    return R


def ref_tt_build(prob, alpha, dt, u=None, du=None, builds=1):
    """Build_M_K_R_SUPG / Build_M_K_R_DD of the reference (by prob.form, with
    prob.cau and prob.h_shock) at (u, du); returns (A[nel, 9], R[neq+1])."""
    m = prob.mesh
    R = ref_tt()
    u = np.zeros(m.neq) if u is None else np.ascontiguousarray(u, dtype=np.float64)
    du = np.zeros(m.neq) if du is None else np.ascontiguousarray(du, dtype=np.float64)
    cau = int(prob.cau)
    R.fr_tt_set_form(int(getattr(prob, "form", 0)), cau if cau in (2, 3) else 1, int(getattr(prob, "h_shock", 0)))
    A = np.empty(m.nel * 9)
    F = np.zeros(m.neq + 1)
    R.fr_tt_build(*_mesh_args(m), prob.k, prob.gamma, prob.beta[0], prob.beta[1], prob.f, prob.upmode, prob.upval,
                  float(alpha), float(dt), u, du, int(builds), A, F)
    return A.reshape(m.nel, 9), F


def _ref_tt_form(R, prob):
    cau = int(prob.cau)
    R.fr_tt_set_form(1, cau if cau in (2, 3) else 2, int(getattr(prob, "h_shock", 0)))


def ref_tt_mfdd_build(prob, alpha, dt, u, du, uB, duB, Da):
    """The reference's Build_M_F_DD (fresh delta_old) at (u, du, uB, duB),
    then its calculate_DaB on Da; returns (A[nel, 9], F[neq+1], cond[nel,
    5], DaB[nel])."""
    m = prob.mesh
    R = ref_tt()
    _ref_tt_form(R, prob)
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    A = np.empty(m.nel * 9)
    F = np.zeros(m.neq + 1)
    cond = np.empty(m.nel * 5)
    DaB = np.empty(m.nel)
    R.fr_tt_mfdd_build(*_mesh_args(m), prob.k, prob.gamma, prob.beta[0], prob.beta[1], prob.f, prob.upmode,
                       prob.upval, float(alpha), float(dt), f(u), f(du), f(uB), f(duB), f(Da), A, F, cond, DaB)
    return A.reshape(m.nel, 9), F, cond.reshape(m.nel, 5), DaB


def ref_tt_predictor1(prob, alpha, dt, topts: TimeOpts, tol=1e-10, kmax=30, lmax=1000, u0=None, dropin=False):
    """The reference's Predictor_Old with Build_M_K_R_SUPG / Build_M_K_R_DD
    (by prob.form), Diag and pgmres; returns (u[neq], GMRES iterations)."""
    m = prob.mesh
    R = ref_tt(dropin)
    cau = int(prob.cau)
    R.fr_tt_set_form(int(getattr(prob, "form", 0)), cau if cau in (2, 3) else 1, int(getattr(prob, "h_shock", 0)))
    perm, inv, _ = permutation_of_lm(m)
    init = np.zeros(m.neq + 1) if u0 is None else np.append(np.asarray(u0, dtype=np.float64), 0.0)
    u = np.zeros(m.neq + 1)
    its = R.fr_tt_predictor1(*_mesh_args(m), prob.k, prob.gamma, prob.beta[0], prob.beta[1], prob.f, prob.upmode,
                             prob.upval, float(alpha), float(dt), perm, inv, init, topts.as_array(), int(kmax),
                             int(lmax), float(tol), u)
    return u[:m.neq].copy(), its


def ref_tt_layout():
    out = np.zeros(64, dtype=np.int64)
    ref_tt().fr_tt_layout(out)
    return out


def ref_tt_predictor2(prob, alpha, dt, topts: TimeOpts, tol=1e-10, kmax=30, lmax=1000, u0=None, dropin=False):
    """The reference's Predictor_New with Build_M_F_DD, Diag and pgmres;
    returns (u[neq], GMRES iterations)."""
    m = prob.mesh
    R = ref_tt(dropin)
    _ref_tt_form(R, prob)
    perm, inv, _ = permutation_of_lm(m)
    init = np.zeros(m.neq + 1) if u0 is None else np.append(np.asarray(u0, dtype=np.float64), 0.0)
    u = np.zeros(m.neq + 1)
    its = R.fr_tt_predictor2(*_mesh_args(m), prob.k, prob.gamma, prob.beta[0], prob.beta[1], prob.f, prob.upmode,
                             prob.upval, float(alpha), float(dt), perm, inv, init, topts.as_array(), int(kmax),
                             int(lmax), float(tol), u)
    return u[:m.neq].copy(), its


def build_tt(prob, alpha, dt, u=None, du=None):
    """Build_M_K_R_SUPG (transient transport) at (u, du); returns
    (A[nel, 9] = me + alpha dt ke, R[neq+1])."""
    m = prob.mesh
    u = np.zeros(m.neq) if u is None else np.ascontiguousarray(u, dtype=np.float64)
    du = np.zeros(m.neq) if du is None else np.ascontiguousarray(du, dtype=np.float64)
    A = np.empty(m.nel * 9)
    R = np.empty(m.neq + 1)
    s, keep = _problem_struct(prob)
    lib().or_build_tt(*_mesh_args(m), ctypes.byref(s), float(alpha), float(dt), u, du, A, R)
    return A.reshape(m.nel, 9), R


def tt_predictor(prob, alpha, dt, topts: TimeOpts, tol=1e-10, kmax=30, lmax=1000, u0=None):
    """Predictor_Old with the transient transport build; returns (u, a, stats)."""
    m = prob.mesh
    u = np.zeros(m.neq + 1)
    if u0 is not None:
        u[:m.neq] = u0
    a = np.zeros(m.neq + 1)
    st = _TimeStats()
    s, keep = _problem_struct(prob)
    lib().or_tt_predictor(*_mesh_args(m), ctypes.byref(s), float(alpha), float(dt), ctypes.byref(topts), tol, kmax,
                          lmax, u, a, ctypes.byref(st))
    return u[:m.neq].copy(), a[:m.neq].copy(), {k: getattr(st, k) for k, _ in st._fields_}


def build_tt_mfdd(prob, alpha, dt, u=None, du=None, uB=None, duB=None, delta_old=None):
    """Build_M_F_DD (TimeIntegration "Predictor2", form DD) at (u, du) with
    the bubble unknowns (uB, duB: one per element); returns (A[nel, 9],
    F[neq+1], cond[nel, 5] = invN2, R2, M2[0..2]).  delta_old (nel, updated
    in place) is the relaxed shock-capture state, None = fresh zeros."""
    m = prob.mesh
    z = np.zeros
    u = z(m.neq) if u is None else np.ascontiguousarray(u, dtype=np.float64)
    du = z(m.neq) if du is None else np.ascontiguousarray(du, dtype=np.float64)
    uB = z(m.nel) if uB is None else np.ascontiguousarray(uB, dtype=np.float64)
    duB = z(m.nel) if duB is None else np.ascontiguousarray(duB, dtype=np.float64)
    A = np.empty(m.nel * 9)
    F = np.empty(m.neq + 1)
    cond = np.empty(m.nel * 5)
    s, keep = _problem_struct(prob)
    if delta_old is not None:
        s.delta_old = delta_old.ctypes.data
    lib().or_build_tt_mfdd(*_mesh_args(m), ctypes.byref(s), float(alpha), float(dt), u, du, uB, duB, A, F, cond)
    return A.reshape(m.nel, 9), F, cond.reshape(m.nel, 5)


def tt_dab(lm, cond, Da):
    """calculate_DaB: the bubble increments (nel) from Da (neq + 1)."""
    nel = lm.shape[0]
    Da = np.array(Da, dtype=np.float64, copy=True)
    DaB = np.empty(nel)
    lib().or_tt_dab(nel, np.ascontiguousarray(lm, dtype=np.int32).reshape(-1), Da.shape[0] - 1,
                    np.ascontiguousarray(cond, dtype=np.float64).reshape(-1), Da, DaB)
    return DaB


def tt_predictor2(prob, alpha, dt, topts: TimeOpts, tol=1e-10, kmax=30, lmax=1000, u0=None):
    """Predictor_New with Build_M_F_DD ("Predictor2", form DD); returns
    (u, a, uB, aB, stats)."""
    m = prob.mesh
    u = np.zeros(m.neq + 1)
    if u0 is not None:
        u[:m.neq] = u0
    a = np.zeros(m.neq + 1)
    uB = np.zeros(max(m.nel, 1))
    aB = np.zeros(max(m.nel, 1))
    st = _TimeStats()
    s, keep = _problem_struct(prob)
    lib().or_tt_predictor2(*_mesh_args(m), ctypes.byref(s), float(alpha), float(dt), ctypes.byref(topts), tol, kmax,
                           lmax, u, a, uB, aB, ctypes.byref(st))
    return (u[:m.neq].copy(), a[:m.neq].copy(), uB[:m.nel].copy(), aB[:m.nel].copy(),
            {k: getattr(st, k) for k, _ in st._fields_})


def ebemv3_perm(lm, A, perm, inv, P):
    nel = lm.shape[0]
    n = perm.shape[0] - 1
    Q = np.zeros(n + 1, dtype=np.float64)
    lib().or_ebemv3_perm(nel, np.ascontiguousarray(lm, dtype=np.int32).reshape(-1),
                         np.ascontiguousarray(A, dtype=np.float64).reshape(-1), perm, inv, n,
                         np.ascontiguousarray(P, dtype=np.float64), Q)
    return Q


def ebemv(lm, A, NEQ, P):
    nel, S = lm.shape
    Q = np.zeros(NEQ + 1, dtype=np.float64)
    lib().or_ebemv(nel, S, np.ascontiguousarray(lm, dtype=np.int32).reshape(-1),
                   np.ascontiguousarray(A, dtype=np.float64).reshape(-1), NEQ,
                   np.ascontiguousarray(P, dtype=np.float64), Q)
    return Q


def diag_setup(lm, A, NEQ, F, Diag=None):
    nel, S = lm.shape
    Diag = np.zeros(NEQ + 1) if Diag is None else Diag
    invDiag = np.zeros(NEQ + 1)
    F = np.array(F, dtype=np.float64, copy=True)
    lib().or_diag_setup(nel, S, np.ascontiguousarray(lm, dtype=np.int32).reshape(-1),
                        np.ascontiguousarray(A, dtype=np.float64).reshape(-1), NEQ, Diag, invDiag, F)
    return Diag, invDiag, F


def blockdiag_setup(mesh, A, F, ref_quirks=True):
    """Nodal block-diagonal setup; returns (BlockDiag, invBlockDiag, Id, F')."""
    B = mesh.ndof
    Id = np.where(mesh.type == 0, mesh.neq, mesh.invp).astype(np.int32)
    bd = np.zeros(mesh.nnodes * B * B)
    ibd = np.zeros(mesh.nnodes * B * B)
    F = np.array(F, dtype=np.float64, copy=True)
    lib().or_blockdiag_setup(mesh.nnodes, mesh.nel, B, np.ascontiguousarray(mesh.ien, dtype=np.int32).reshape(-1),
                             np.ascontiguousarray(A, dtype=np.float64).reshape(-1), Id, mesh.neq,
                             int(ref_quirks), bd, ibd, F)
    return bd, ibd, Id, F


def blockdiag_apply(mesh, ibd, Id, p):
    p = np.array(p, dtype=np.float64, copy=True)
    z = np.zeros_like(p)
    lib().or_blockdiag_apply(mesh.nnodes, mesh.ndof, Id, mesh.neq, ibd, p, z)
    return z


def ebe_diag_solve(lm, A, NEQ, F, perm=None, inv=None, Diag=None, kmax=30, lmax=1000, tol=1e-10):
    """Diag setup + pgmres; returns (X, iterations, Diag, invDiag, F')."""
    nel, S = lm.shape
    Diag = np.zeros(NEQ + 1) if Diag is None else Diag
    invDiag = np.zeros(NEQ + 1)
    F = np.array(F, dtype=np.float64, copy=True)
    X = np.zeros(NEQ + 1)
    pp = perm.ctypes.data if perm is not None else None
    ip = inv.ctypes.data if inv is not None else None
    it = lib().or_ebe_diag_solve(nel, S, np.ascontiguousarray(lm, dtype=np.int32).reshape(-1),
                                 np.ascontiguousarray(A, dtype=np.float64).reshape(-1), NEQ,
                                 pp, ip, Diag, invDiag, F, kmax, lmax, tol, X)
    return X, it, Diag, invDiag, F


# ---- element preconditioners "LUe" (kind 1) and "SGSe" (kind 2) ----
def _lmA(lm, A):
    return (np.ascontiguousarray(lm, dtype=np.int32).reshape(-1), np.ascontiguousarray(A, dtype=np.float64).reshape(-1))


def elem_prec_apply(kind, lm, A, NEQ, z):
    """kind 1: LUe set-up + LU_precond_EBE; 2: the SGS forward sweep; 3: the
    SGS backward sweep (SGS_precondR_EBE); z (NEQ+1) not modified."""
    l, a = _lmA(lm, A)
    nel = lm.shape[0]
    z = np.array(z, dtype=np.float64, copy=True)
    if kind == 1:
        LUe = np.zeros(9 * nel)
        lib().or_lue_setup(nel, a, LUe)
        lib().or_lue_apply(nel, l, NEQ, LUe, z)
    elif kind == 2:
        lib().or_sgs_fwd(nel, l, NEQ, a, z)
    else:
        lib().or_sgs_bwd(nel, l, NEQ, a, z)
    return z


def ebe_elem_solve(kind, lm, A, NEQ, F, perm=None, inv=None, kmax=30, lmax=1000, tol=1e-10):
    """Element-preconditioner set-up + pgmres (kind 1 LUe, 2 SGSe);
    returns (X, iterations, F')."""
    l, a = _lmA(lm, A)
    F = np.array(F, dtype=np.float64, copy=True)
    X = np.zeros(NEQ + 1)
    pp = perm.ctypes.data if perm is not None else None
    ip = inv.ctypes.data if inv is not None else None
    it = lib().or_ebe_elem_solve(kind, lm.shape[0], l, a, NEQ, pp, ip, F, kmax, lmax, tol, X)
    return X, it, F


def ref_elem_prec_apply(kind, lm, A, NEQ, z):
    l, a = _lmA(lm, A)
    z = np.array(z, dtype=np.float64, copy=True)
    ref().fr_ebe_prec_apply(kind, lm.shape[0], NEQ, l, a, z)
    return z


def ref_ebe_elem_solve(kind, lm, A, perm, inv, F, kmax=30, lmax=1000, tol=1e-10):
    l, a = _lmA(lm, A)
    n = perm.shape[0] - 1
    F = np.array(F, dtype=np.float64, copy=True)
    X = np.zeros(n + 1)
    it = ref().fr_ebe_prec_pgmres(kind, lm.shape[0], n, l, a, perm, inv, F, X, kmax, lmax, tol)
    return X, it, F


def ebe_block_solve(mesh, A, F, kmax=30, lmax=1000, tol=1e-10, ref_quirks=True):
    """Nodal block-diagonal set-up + pgmres on EBE blocks; returns (X, iterations, F')."""
    B = mesh.ndof
    Id = np.where(mesh.type == 0, mesh.neq, mesh.invp).astype(np.int32)
    F = np.array(F, dtype=np.float64, copy=True)
    X = np.zeros(mesh.neq + 1)
    lm = fill_lm(mesh)
    it = lib().or_ebe_block_solve(mesh.nnodes, mesh.nel, B, np.ascontiguousarray(mesh.ien, dtype=np.int32).reshape(-1),
                                  np.ascontiguousarray(lm, dtype=np.int32).reshape(-1),
                                  np.ascontiguousarray(A, dtype=np.float64).reshape(-1), Id, mesh.neq,
                                  int(ref_quirks), F, kmax, lmax, tol, X)
    return X, it, F


def transport_process(prob, solver_tol=1e-10, nonlinear_tol=1e-3, kmax=30, lmax=1000, max_nonlinear=1000):
    """Steady transport Process loop; returns (U[neq], nonlinear its, GMRES its)."""
    m = prob.mesh
    U = np.zeros(m.neq + 1)
    its = _c_int(0)
    s, keep = _problem_struct(prob)
    nl = lib().or_transport_process(*_mesh_args(m), ctypes.byref(s), solver_tol, nonlinear_tol,
                                    kmax, lmax, max_nonlinear, U, ctypes.byref(its))
    return U[:m.neq].copy(), nl, its.value


# ------------------------------------------------------- reference build
def ref_connectivity(mesh):
    R = ref()
    n = mesh.neq
    lm = np.empty(mesh.nel * 3, dtype=np.int32)
    perm = np.empty(n + 1, dtype=np.int32)
    inv = np.empty(n + 1, dtype=np.int32)
    band = np.zeros(2, dtype=np.int32)
    nnz = R.fr_sst_connectivity(*_mesh_args(mesh), lm, perm, inv, band)
    return lm.reshape(mesh.nel, 3), perm, inv, band, nnz


def _ref_form(prob, R=None):
    """StabilizationForm / ShockCapture of the reference run: "SUPG" or "DD",
    "CAU" (cau 1, and the reference's stand-in for cau 0) or "CAUDD"."""
    (R or ref()).fr_sst_set_form(int(getattr(prob, "form", 0)), int(prob.cau) if int(prob.cau) in (2, 3) else 1,
                          int(getattr(prob, "h_shock", 0)))


def ref_build(prob, u=None):
    m = prob.mesh
    if u is None:
        u = np.zeros(m.neq)
    A = np.empty(m.nel * 9)
    F = np.empty(m.neq + 1)
    F[m.neq] = 0.0
    _ref_form(prob)
    ref().fr_sst_build(*_mesh_args(m), prob.k, prob.gamma, prob.beta[0], prob.beta[1], prob.f,
                       prob.upmode, prob.upval, np.ascontiguousarray(u, dtype=np.float64), A, F)
    return A.reshape(m.nel, 9), F


def ref_process(prob, solver_tol=1e-10, nonlinear_tol=1e-3, kmax=30, lmax=1000, dropin=False):
    """The reference's Process loop (dropin: its drop-in build, the same
    driver on the library's GPU solve path)."""
    m = prob.mesh
    U = np.zeros(m.neq + 1)
    its = _c_int(0)
    R = ref(DROPIN_SO["sst"]) if dropin else ref()
    _ref_form(prob, R)
    R.fr_sst_process(*_mesh_args(m), prob.k, prob.gamma, prob.beta[0], prob.beta[1], prob.f,
                         prob.upmode, prob.upval, solver_tol, nonlinear_tol, kmax, lmax, U, ctypes.byref(its))
    return U[:m.neq].copy(), its.value


def ref_timed_solve(prob, kmax=30, lmax=1000, tol=1e-10):
    """One iteration of the reference's Process (Build_K_F at u = 0,
    scaling, Diag set-up, pgmres, unscaling), timed inside the reference
    build after its untimed Preprocess work; returns (seconds, GMRES
    iterations)."""
    m = prob.mesh
    sec = _c_dbl(0.0)
    R = ref()
    _ref_form(prob, R)
    its = R.fr_sst_timed_solve(*_mesh_args(m), prob.k, prob.gamma, prob.beta[0], prob.beta[1], prob.f,
                               prob.upmode, prob.upval, int(kmax), int(lmax), float(tol), ctypes.byref(sec))
    return sec.value, its


def ref_ebemv(lm, A, perm, inv, P):
    nel = lm.shape[0]
    n = perm.shape[0] - 1
    Q = np.zeros(n + 1)
    ref().fr_ebemv(nel, n, np.ascontiguousarray(lm, dtype=np.int32).reshape(-1),
                   np.ascontiguousarray(A, dtype=np.float64).reshape(-1), perm, inv,
                   np.ascontiguousarray(P, dtype=np.float64), Q)
    return Q


def ref_diag_pgmres(lm, A, perm, inv, F, kmax=30, lmax=1000, tol=1e-10, Diag=None):
    nel = lm.shape[0]
    n = perm.shape[0] - 1
    Diag = np.zeros(n + 1) if Diag is None else Diag
    invDiag = np.zeros(n + 1)
    F = np.array(F, dtype=np.float64, copy=True)
    X = np.zeros(n + 1)
    it = ref().fr_diag_pgmres(nel, n, np.ascontiguousarray(lm, dtype=np.int32).reshape(-1),
                              np.ascontiguousarray(A, dtype=np.float64).reshape(-1), perm, inv,
                              Diag, invDiag, F, X, kmax, lmax, tol)
    return X, it, Diag, invDiag, F


def ref_symrcm(IA, JA):
    n = IA.shape[0] - 1
    p = np.empty(max(n, 1), dtype=np.int32)
    ref().fr_symrcm(n, int(IA[-1]), np.array(IA, dtype=np.int32), np.array(JA, dtype=np.int32), p)
    return p[:n]


def ref_layout():
    out = np.zeros(64, dtype=np.int64)
    ref().fr_sst_layout(out)
    return out


# ------------------------------------------------------- CSR path and ILU(0)
def csr_pattern(mesh, perm, inv):
    """CSR pattern of the free dofs in the RCM numbering of csr_Initialization."""
    L = lib()
    L.or_csr_pattern.argtypes = [_c_int, _i32p, _i32p, _i32p, _c_int, _i32p, _i32p, _i32p, _i32p]
    n = mesh.neq
    IA = np.empty(n + 1, dtype=np.int32)
    JA = np.empty(mesh.nel * 9 * mesh.ndof ** 2 + 1, dtype=np.int32)
    nnz = L.or_csr_pattern(mesh.nel, np.ascontiguousarray(mesh.ien, dtype=np.int32).reshape(-1),
                           mesh.type, mesh.invp, n, perm, inv, IA, JA)
    return IA, JA[:nnz].copy()


def csr_assemble(lm_new, A, NEQ, IA, JA):
    L = lib()
    L.or_csr_assemble.argtypes = [_c_int, _c_int, _i32p, _f64p, _c_int, _i32p, _i32p, _f64p]
    L.or_csr_assemble.restype = None
    nel, S = lm_new.shape
    AA = np.zeros(JA.shape[0])
    L.or_csr_assemble(nel, S, np.ascontiguousarray(lm_new, dtype=np.int32).reshape(-1),
                      np.ascontiguousarray(A, dtype=np.float64).reshape(-1), NEQ, IA, JA, AA)
    return AA


def csrmv(IA, JA, AA, P):
    L = lib()
    L.or_csrmv.argtypes = [_c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
    L.or_csrmv.restype = None
    n = IA.shape[0] - 1
    Q = np.zeros(n + 1)
    L.or_csrmv(n, IA, JA, AA, np.ascontiguousarray(P, dtype=np.float64), Q)
    return Q


def ilu0(IA, JA, AA):
    L = lib()
    L.or_ilu0_factor.argtypes = [_c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
    n = IA.shape[0] - 1
    LU = np.zeros_like(AA)
    D = np.zeros(n)
    rc = L.or_ilu0_factor(n, IA, JA, AA, LU, D)
    return rc, LU, D


def ilu0_apply(IA, JA, LU, D, y):
    L = lib()
    L.or_ilu0_apply.argtypes = [_c_int, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p]
    L.or_ilu0_apply.restype = None
    n = IA.shape[0] - 1
    x = np.zeros(n + 1)
    L.or_ilu0_apply(n, IA, JA, LU, D, np.ascontiguousarray(y, dtype=np.float64), x)
    return x


def ilup(IA, JA, AA, p):
    """ILU(p): returns (FIA, FJA, FDG, LU, D) on the factor CSR."""
    L = lib()
    n = len(IA) - 1
    IA = np.ascontiguousarray(IA, dtype=np.int32)
    JA = np.ascontiguousarray(JA, dtype=np.int32)
    pi = ctypes.POINTER(_c_int)
    fia, fja, fdg = pi(), pi(), pi()
    L.or_ilup_symbolic.argtypes = [_c_int, _i32p, _i32p, _c_int, ctypes.POINTER(pi), ctypes.POINTER(pi),
                                   ctypes.POINTER(pi)]
    L.or_ilup_symbolic(n, IA, JA, int(p), ctypes.byref(fia), ctypes.byref(fja), ctypes.byref(fdg))
    FIA = np.ctypeslib.as_array(fia, shape=(n + 1,)).copy()
    FJA = np.ctypeslib.as_array(fja, shape=(max(int(FIA[-1]), 1),)).copy()[: int(FIA[-1])]
    FDG = np.ctypeslib.as_array(fdg, shape=(max(n, 1),)).copy()[:n]
    libc = ctypes.CDLL(None)
    libc.free.argtypes = [ctypes.c_void_p]
    for q in (fia, fja, fdg):
        libc.free(ctypes.cast(q, ctypes.c_void_p))
    LU = np.zeros(max(int(FIA[-1]), 1))
    D = np.zeros(max(n, 1))
    L.or_ilup_factor.argtypes = [_c_int, _i32p, _i32p, _f64p, _i32p, _i32p, _i32p, _f64p, _f64p]
    rc = L.or_ilup_factor(n, IA, JA, np.ascontiguousarray(AA, dtype=np.float64), FIA, FJA, FDG, LU, D)
    if rc:
        raise ZeroDivisionError(f"ILU({p}): zero pivot in row {rc - 1}")
    return FIA, FJA, FDG, LU, D


def block_diagonal_csr(IA, JA, AA, blocks):
    """The couplings among the rows of each of `blocks` equal row blocks
    (rows q n / P .. (q+1) n / P - 1): the CSR block each MPI rank of the
    reference factorises by itself (CSR/ILUp_precond_setup.c:20-29, the
    rank's own rows and columns).  Returns (IA, JA, AA) of that matrix."""
    IA = np.asarray(IA)
    JA = np.asarray(JA)
    AA = np.asarray(AA)
    n = len(IA) - 1
    blk = np.empty(n, dtype=np.int64)
    for q in range(blocks):
        blk[q * n // blocks:(q + 1) * n // blocks] = q
    rows = np.repeat(np.arange(n), np.diff(IA))
    keep = blk[JA[:IA[-1]]] == blk[rows]
    BIA = np.concatenate([[0], np.cumsum(np.bincount(rows[keep], minlength=n))]).astype(np.int32)
    return BIA, JA[:IA[-1]][keep].astype(np.int32), AA[:IA[-1]][keep].astype(np.float64)


def ilup_apply(FIA, FJA, FDG, LU, D, y):
    L = lib()
    n = len(FIA) - 1
    L.or_ilup_apply.argtypes = [_c_int, _i32p, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p]
    L.or_ilup_apply.restype = None
    x = np.zeros(n)
    L.or_ilup_apply(n, FIA, FJA, FDG, LU, D, np.ascontiguousarray(y[:n], dtype=np.float64), x)
    return x


def ref_csr(prob, A, P, ilu_p=0):
    """The reference's csr_Initialization + csr_assembly + csrmv + ILU(p)
    (Preconditioner "ILU<p>"): z = M^-1 P."""
    R = ref()
    R.fr_sst_set_ilu.argtypes = [_c_int]
    R.fr_sst_set_ilu.restype = None
    R.fr_sst_set_ilu(int(ilu_p))
    R.fr_sst_csr.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int, _f64p, _c_int,
                             _i32p, _i32p, _f64p, _i32p, _f64p, _f64p, _f64p]
    m = prob.mesh
    nmax = m.nel * 9 + 1
    IA = np.empty(m.neq + 1, dtype=np.int32)
    JA = np.empty(nmax, dtype=np.int32)
    AA = np.empty(nmax)
    invp = np.empty(m.nnodes, dtype=np.int32)
    Q = np.zeros(m.neq + 1)
    z = np.zeros(m.neq + 1)
    nnz = R.fr_sst_csr(*_mesh_args(m), np.ascontiguousarray(A, dtype=np.float64).reshape(-1), nmax, IA, JA, AA,
                       invp, np.ascontiguousarray(P, dtype=np.float64), Q, z)
    return IA, JA[:nnz].copy(), AA[:nnz].copy(), invp, Q, z


class Spike:
    """Truncated SPIKE (oracle/spike.c) of a CSR matrix (IA, JA, AA, 0-based,
    internal numbering): `apply(f)` returns M^-1 f for n-entry f."""

    def __init__(self, IA, JA, AA, k, parts):
        L = lib()
        L.or_spike_setup.argtypes = [_c_int, _i32p, _i32p, _f64p, _c_int, _c_int, ctypes.POINTER(ctypes.c_int)]
        L.or_spike_setup.restype = ctypes.c_void_p
        L.or_spike_apply.argtypes = [ctypes.c_void_p, _f64p, _f64p]
        L.or_spike_apply.restype = None
        L.or_spike_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), _i32p, _i32p, _i32p]
        L.or_spike_free.argtypes = [ctypes.c_void_p]
        L.or_spike_free.restype = None
        self._L = L
        self.n = int(IA.shape[0]) - 1
        err = ctypes.c_int(0)
        self._h = L.or_spike_setup(self.n, np.ascontiguousarray(IA, dtype=np.int32),
                                   np.ascontiguousarray(JA, dtype=np.int32),
                                   np.ascontiguousarray(AA, dtype=np.float64), int(k), int(parts), ctypes.byref(err))
        self.err = err.value
        if not self._h:
            raise ValueError("or_spike_setup rejected its arguments")
        kk = ctypes.c_int(0)
        nb = L.or_spike_blocks(self.n, int(k), int(parts))
        self.bs = np.zeros(nb + 1, np.int32)
        self.kl = np.zeros(nb, np.int32)
        self.ku = np.zeros(nb, np.int32)
        P = L.or_spike_info(self._h, ctypes.byref(kk), self.bs, self.kl, self.ku)
        self.P, self.k = P, kk.value

    def apply(self, f):
        f = np.ascontiguousarray(f[: self.n], dtype=np.float64)
        y = np.zeros(self.n)
        self._L.or_spike_apply(self._h, f, y)
        return y

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.or_spike_free(self._h)
            self._h = None


def scale(lm, A, NEQ, F, kind, Diag=None):
    """Left ("Left") or LeftRight ("LeftRight") scaling of an EBE system;
    returns (A scaled, F scaled, Diag, invDiag[NEQ+1])."""
    L = lib()
    fn = L.or_scale_left if kind == "Left" else L.or_scale_leftright
    fn.argtypes = [_c_int, _c_int, _i32p, _f64p, _c_int, _f64p, _f64p, _f64p]
    fn.restype = None
    nel, S = lm.shape
    A = np.array(A, dtype=np.float64, copy=True).reshape(-1)
    F = np.array(F, dtype=np.float64, copy=True)
    D = np.zeros(NEQ + 1) if Diag is None else np.array(Diag, dtype=np.float64, copy=True)
    inv = np.zeros(NEQ + 1)
    fn(nel, S, np.ascontiguousarray(lm, dtype=np.int32).reshape(-1), A, NEQ, D, inv, F)
    return A.reshape(nel, S * S), F, D, inv


def unscale(invDiag, x):
    L = lib()
    L.or_unscale.argtypes = [_c_int, _f64p, _f64p]
    L.or_unscale.restype = None
    x = np.array(x, dtype=np.float64, copy=True)
    L.or_unscale(invDiag.shape[0] - 1, np.ascontiguousarray(invDiag, dtype=np.float64), x)
    return x




def block_scale(mesh, A, inv, B=4):
    """Block_scaling_EBE's element-block part (oracle/ebe_gmres.c) on copies:
    returns the scaled blocks (nel, (3B)^2)."""
    L = lib()
    L.or_block_scale.argtypes = [_c_int, _c_int, _i32p, _i32p, _c_int, _f64p, _f64p]
    L.or_block_scale.restype = None
    Id = np.where(mesh.type == 0, mesh.neq, mesh.invp).astype(np.int32)
    Ac = np.array(A, dtype=np.float64, copy=True).reshape(-1)
    L.or_block_scale(mesh.nel, B, np.ascontiguousarray(mesh.ien, dtype=np.int32).reshape(-1), Id, mesh.neq,
                     np.ascontiguousarray(inv, dtype=np.float64).reshape(-1), Ac)
    return Ac.reshape(mesh.nel, -1)


def ref_euler_block_scale(mesh, A, F):
    """The reference's Block_scaling_EBE: returns (A, F, inverse blocks)."""
    R = ref_euler()
    R.fr_eu_block_scale.argtypes = [_c_int, _c_int, _f64p, _f64p, _i32p, _i32p, _i32p, _c_int, _f64p, _f64p, _f64p]
    R.fr_eu_block_scale.restype = None
    Ac = np.array(A, dtype=np.float64, copy=True).reshape(-1)
    Fc = np.array(F, dtype=np.float64, copy=True)
    inv = np.empty(mesh.nnodes * 16)
    R.fr_eu_block_scale(*_mesh_args(mesh), Ac, Fc, inv)
    return Ac.reshape(mesh.nel, 144), Fc, inv
