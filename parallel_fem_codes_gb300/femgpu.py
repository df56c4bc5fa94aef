"""ctypes binding of libfemgpu (include/femgpu.h) and a thin object layer.

The library is loaded from the package's in-tree build
(parallel_fem_codes_gb300/_lib/libfemgpu.so).  There is no fallback: if the
library is missing or a call fails, an exception says why.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os

import numpy as np

from . import build as _build

FG_OK = 0
FG_PRECOND_NONE, FG_PRECOND_DIAG, FG_PRECOND_BLOCKDIAG, FG_PRECOND_ILU0, FG_PRECOND_SPIKE = 0, 1, 2, 3, 4
FG_PRECOND_LUE, FG_PRECOND_SGSE = 5, 6   # element LU sweep ("LUe"); element SGS ("SGSe", right sweep too)
FG_SCALE_LEFT, FG_SCALE_LEFTRIGHT, FG_SCALE_BLOCK = 1, 2, 3
FG_OP_EBE, FG_OP_CSR = 0, 1
FG_SETUP_ACCUMULATE, FG_SETUP_REF_QUIRKS = 1, 2
FG_PREC_FP64, FG_PREC_MIXED, FG_PREC_MIXED16 = 64, 32, 16
FG_TIME_PREDICTOR, FG_TIME_BDF, FG_TIME_TRBDF2, FG_TIME_PREDICTOR2 = 0, 1, 2, 3
FG_TIME_PREDICTOR2_BDF, FG_TIME_PREDICTOR2_TRBDF2 = 4, 5
FG_NS_SUPG_PSPG, FG_NS_VMS_DCDD = 0, 1
FG_TRANSPORT_SUPG, FG_TRANSPORT_DD = 0, 1
FG_EULER_SUPG, FG_EULER_DD = 0, 1
FG_SHOCK_NONE, FG_SHOCK_CAU, FG_SHOCK_CAUDD, FG_SHOCK_YZBETA = 0, 1, 2, 3
FG_HSHOCK_2SQRTAREA, FG_HSHOCK_OPTION1, FG_HSHOCK_OPTION2 = 0, 1, 2
FG_REORDER_NONE, FG_REORDER_RCM = 0, 1
FG_ERR_ARG, FG_ERR_CUDA, FG_ERR_NOMEM, FG_ERR_STATE = 1, 2, 3, 4
FG_ERR_BREAKDOWN, FG_ERR_NOTCONV, FG_ERR_UNSUPPORTED, FG_ERR_TIMEOUT = 5, 6, 7, 8
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_NOMEM", 4: "ERR_STATE",
          5: "ERR_BREAKDOWN", 6: "ERR_NOTCONV", 7: "ERR_UNSUPPORTED", 8: "ERR_TIMEOUT"}

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_c_int, _c_dbl = ctypes.c_int, ctypes.c_double


class FemGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class SystemInfo(ctypes.Structure):
    _fields_ = [("n", _c_int), ("nel", _c_int), ("ndof", _c_int), ("S", _c_int), ("nnodes", _c_int),
                ("ncolours", _c_int), ("bandwidth_before", _c_int), ("bandwidth_after", _c_int),
                ("nnz", _c_int), ("device_bytes", ctypes.c_size_t)]


class SolverOpts(ctypes.Structure):
    _fields_ = [("kmax", _c_int), ("lmax", _c_int), ("tol", _c_dbl), ("precision", _c_int),
                ("inner_tol", _c_dbl)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", _c_int), ("cycles", _c_int), ("converged", _c_int), ("status", _c_int),
                ("rho", _c_dbl), ("eps", _c_dbl), ("true_rel_residual", _c_dbl), ("seconds", _c_dbl)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TransportCoeffs(ctypes.Structure):
    _fields_ = [("k", _c_dbl), ("gamma", _c_dbl), ("beta", _c_dbl * 2), ("f", _c_dbl), ("cau", _c_int),
                ("form", _c_int), ("h_shock", _c_int)]


class TTCoeffs(ctypes.Structure):
    """fg_tt_coeffs: transport coefficients plus Alpha and DeltaT."""
    _fields_ = [("c", TransportCoeffs), ("alpha", _c_dbl), ("dt", _c_dbl)]


class MeshInfo(ctypes.Structure):
    _fields_ = [("nnodes", _c_int), ("nel", _c_int), ("neq", _c_int)]


class ProcessStats(ctypes.Structure):
    _fields_ = [("nonlinear_iterations", _c_int), ("gmres_iterations", _c_int), ("seconds", _c_dbl),
                ("true_rel_residual", _c_dbl), ("nonlinear_residual", _c_dbl)]


class NSCoeffs(ctypes.Structure):
    _fields_ = [("reynolds", _c_dbl), ("precond", _c_int), ("form", _c_int)]


class EulerCoeffs(ctypes.Structure):
    _fields_ = [("gamma", _c_dbl), ("mach", _c_dbl), ("dimensionless", _c_int), ("tolerance", _c_dbl),
                ("alpha", _c_dbl), ("dt", _c_dbl), ("form", _c_int), ("invY", _c_dbl * 4), ("shock", _c_int)]


class TimeOpts(ctypes.Structure):
    _fields_ = [("stop_by_norm", _c_int), ("max_corrections", _c_int), ("correction_tol", _c_dbl),
                ("steady_state", _c_int), ("final_time", _c_dbl), ("time_tol", _c_dbl), ("max_steps", _c_int),
                ("precond", _c_int), ("setup_flags", _c_int), ("scheme", _c_int)]


class TimeStats(ctypes.Structure):
    _fields_ = [("steps", _c_int), ("corrections", _c_int), ("gmres_iterations", _c_int), ("t", _c_dbl),
                ("seconds", _c_dbl), ("true_rel_residual", _c_dbl)]


class TuneChoice(ctypes.Structure):
    _fields_ = [("part_dofs", _c_int), ("mv3_pipeline", _c_int), ("ms_per_cycle", _c_dbl),
                ("from_cache", _c_int), ("candidates", _c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerOpts(ctypes.Structure):
    _fields_ = [("kmax", _c_int), ("lmax", _c_int), ("tol", _c_dbl), ("precision", _c_int),
                ("inner_tol", _c_dbl), ("hbm_budget_bytes", ctypes.c_size_t), ("max_active", _c_int)]


class ServerResult(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_ulonglong), ("stats", SolveStats), ("t_submit", _c_dbl), ("t_admit", _c_dbl),
                ("t_done", _c_dbl)]

    def as_dict(self):
        return {"tag": self.tag, **self.stats.as_dict(), "t_submit": self.t_submit, "t_admit": self.t_admit,
                "t_done": self.t_done}


_lib = None


def library_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """The loaded libfemgpu; builds it in-tree first when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise FemGpuError(7, f"libfemgpu is not built ({path}); run __graft_entry__.build()")
        _build.build()
    L = ctypes.CDLL(path)
    L.fg_last_error.restype = ctypes.c_char_p
    L.fg_system_create.argtypes = [ctypes.POINTER(_vp), _c_int, _c_int, _c_int, _i32p, _i32p, _i32p, _c_int, _c_int]
    L.fg_system_destroy.argtypes = [_vp]
    L.fg_mesh_analyze.argtypes = [_c_int, _c_int, _c_int, _i32p, _i32p, _i32p, _c_int, _c_int,
                                  _vp, _vp, _vp, _vp, ctypes.POINTER(SystemInfo)]
    L.fg_system_get_info.argtypes = [_vp, ctypes.POINTER(SystemInfo)]
    L.fg_system_get_lm.argtypes = [_vp, _i32p]
    L.fg_system_get_perm.argtypes = [_vp, _i32p, _i32p]
    L.fg_system_get_colours.argtypes = [_vp, _i32p]
    L.fg_set_blocks.argtypes = [_vp, _f64p]
    L.fg_get_blocks.argtypes = [_vp, _f64p]
    L.fg_matvec.argtypes = [_vp, _f64p, _f64p, _c_int]
    L.fg_precond_setup.argtypes = [_vp, _c_int, _c_int, _vp]
    L.fg_precond_apply.argtypes = [_vp, _f64p, _f64p]
    L.fg_precond_apply_right.argtypes = [_vp, _f64p, _f64p]
    L.fg_get_diag.argtypes = [_vp, _f64p]
    L.fg_set_diag.argtypes = [_vp, _f64p]
    L.fg_solve.argtypes = [_vp, ctypes.POINTER(SolverOpts), _f64p, _f64p, _vp, ctypes.POINTER(SolveStats)]
    L.fg_set_geometry.argtypes = [_vp, _f64p, _f64p, _f64p]
    L.fg_transport_assemble.argtypes = [_vp, ctypes.POINTER(TransportCoeffs), _vp, _vp]
    L.fg_solve_batch.argtypes = [_vp, _c_int, ctypes.POINTER(SolverOpts), _vp, _vp, _vp, _vp]
    L.fg_solve_resident.argtypes = [_vp, _c_int, ctypes.POINTER(SolverOpts), _vp]
    L.fg_get_solution.argtypes = [_vp, _f64p]
    L.fg_launch_count.restype = ctypes.c_longlong
    L.fg_set_operator.argtypes = [_vp, _c_int]
    L.fg_set_spike.argtypes = [_vp, _c_int, _c_int]
    L.fg_set_ilu_fill.argtypes = [_vp, _c_int]
    L.fg_set_ilu_blocks.argtypes = [_vp, _c_int]
    L.fg_set_wait_limit.argtypes = [ctypes.c_longlong]
    L.fg_set_memory_limit.argtypes = [ctypes.c_size_t]
    L.fg_autotune.argtypes = [_vp, _c_int, ctypes.POINTER(SolverOpts), _c_int, ctypes.POINTER(TuneChoice)]
    L.fg_tune_lookup.argtypes = [_vp, _c_int, ctypes.POINTER(SolverOpts), ctypes.POINTER(TuneChoice)]
    L.fg_tune_set.argtypes = [_vp, _c_int, ctypes.POINTER(SolverOpts), ctypes.POINTER(TuneChoice)]
    L.fg_tune_clear.restype = None
    L.fg_memory_in_use.restype = ctypes.c_size_t
    L.fg_get_csr.argtypes = [_vp, ctypes.POINTER(_c_int), _vp, _vp, _vp]
    L.fg_system_stream.argtypes = [_vp]
    L.fg_system_stream.restype = _vp
    L.fg_bench_matvec.argtypes = [_vp, _c_int, _c_int, _c_int, ctypes.POINTER(_c_dbl), ctypes.POINTER(_c_dbl)]
    L.fg_transport_prepare.argtypes = [_vp, ctypes.POINTER(TransportCoeffs), _vp]
    L.fg_transport_process.argtypes = [_vp, ctypes.POINTER(TransportCoeffs), ctypes.POINTER(SolverOpts), _c_dbl,
                                       _c_int, _f64p, ctypes.POINTER(ProcessStats)]
    L.fg_ns_set_geometry.argtypes = [_vp, _f64p, _f64p, _f64p, _vp, _vp]
    L.fg_ns_assemble.argtypes = [_vp, ctypes.POINTER(NSCoeffs), _vp, _vp]
    L.fg_ns_process.argtypes = [_vp, ctypes.POINTER(NSCoeffs), ctypes.POINTER(SolverOpts), _c_dbl, _c_int, _f64p,
                                ctypes.POINTER(ProcessStats)]
    L.fg_euler_set_geometry.argtypes = [_vp, _f64p, _f64p, _f64p]
    L.fg_euler_assemble.argtypes = [_vp, ctypes.POINTER(EulerCoeffs), _vp, _vp, _vp]
    L.fg_euler_predictor.argtypes = [_vp, ctypes.POINTER(EulerCoeffs), ctypes.POINTER(SolverOpts),
                                     ctypes.POINTER(TimeOpts), _f64p, _vp, ctypes.POINTER(TimeStats)]
    for name in ("fg_mesh_read", "fg_mesh_read_rank"):
        getattr(L, name).argtypes = [ctypes.c_char_p, _c_int, ctypes.POINTER(MeshInfo), _vp, _vp, _vp, _vp, _vp]
    L.fg_write_vtu.argtypes = [ctypes.c_char_p, _c_int, _c_int, _vp, _vp, _vp, _c_int, _vp, _vp]
    L.fg_scale.argtypes = [_vp, _c_int, _vp]
    L.fg_unscale.argtypes = [_vp, _vp]
    L.fg_tt_assemble.argtypes = [_vp, ctypes.POINTER(TTCoeffs), _vp, _vp, _vp]
    L.fg_tt_bubble_assemble.argtypes = [_vp, ctypes.POINTER(TTCoeffs), _vp, _vp, _vp, _vp, _vp, _vp]
    L.fg_euler_bubble_assemble.argtypes = [_vp, ctypes.POINTER(EulerCoeffs), _vp, _vp, _vp, _vp, _vp, _vp]
    L.fg_bubble_dab.argtypes = [_vp, _vp, _vp]
    L.fg_bubble_state.argtypes = [_vp, _vp, _vp]
    L.fg_tt_predictor.argtypes = [_vp, ctypes.POINTER(TTCoeffs), ctypes.POINTER(SolverOpts),
                                  ctypes.POINTER(TimeOpts), _f64p, _vp, ctypes.POINTER(TimeStats)]
    L.fg_server_create.argtypes = [ctypes.POINTER(_vp), ctypes.POINTER(ServerOpts)]
    L.fg_server_submit.argtypes = [_vp, _vp, ctypes.POINTER(TransportCoeffs), ctypes.c_ulonglong]
    L.fg_server_submit_host.argtypes = [_vp, _vp, _f64p, _f64p, _f64p, ctypes.c_ulonglong]
    L.fg_server_submit_euler.argtypes = [_vp, _vp, ctypes.POINTER(EulerCoeffs), ctypes.POINTER(TimeOpts), _f64p,
                                         ctypes.c_ulonglong]
    L.fg_server_poll.argtypes = [_vp, _vp, _c_int, ctypes.POINTER(_c_int)]
    L.fg_server_wait.argtypes = [_vp, _c_int, _c_dbl]
    L.fg_server_now.argtypes = [_vp]
    L.fg_server_now.restype = _c_dbl
    L.fg_server_destroy.argtypes = [_vp]
    _lib = L
    return L


def check(code: int) -> None:
    if code != FG_OK:
        raise FemGpuError(code, lib().fg_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data


def read_mesh(path, ndof=1, rank_file=False):
    """A mesh file of the reference through the library's reader: a global
    mesh as the structured mesh generator writes it, or (rank_file=True) a
    one-rank partition file.  Returns a meshgen.Mesh."""
    from . import meshgen
    fn = lib().fg_mesh_read_rank if rank_file else lib().fg_mesh_read
    info = MeshInfo()
    p = os.fsencode(path)
    check(fn(p, ndof, ctypes.byref(info), None, None, None, None, None))
    x, y = np.empty(info.nnodes), np.empty(info.nnodes)
    t = np.empty(info.nnodes * ndof, dtype=np.int32)
    iv = np.empty(info.nnodes * ndof, dtype=np.int32)
    ien = np.empty(info.nel * 3, dtype=np.int32)
    check(fn(p, ndof, ctypes.byref(info), x.ctypes.data, y.ctypes.data, t.ctypes.data, iv.ctypes.data,
             ien.ctypes.data))
    return meshgen.Mesh(x=x, y=y, ien=ien.reshape(-1, 3), ndof=ndof, type=t, invp=iv, neq=info.neq)


class _VtuField(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("ncomp", ctypes.c_int), ("values", ctypes.c_void_p)]


def write_vtu(path, mesh, fields, z=None):
    """Paraview output: `fields` maps a name to node values (nnodes) or
    (nnodes, ncomp) with ncomp <= 3, written in order; `z` lifts the points."""
    keep = []
    arr = (_VtuField * max(len(fields), 1))()
    for k, (name, vals) in enumerate(fields.items()):
        v = np.ascontiguousarray(vals, dtype=np.float64)
        if v.shape[0] != mesh.nnodes:
            raise ValueError(f"field {name}: {v.shape[0]} values for {mesh.nnodes} nodes")
        keep.append(v)
        arr[k] = _VtuField(name.encode(), 1 if v.ndim == 1 else v.shape[1], v.ctypes.data)
    x = np.ascontiguousarray(mesh.x, dtype=np.float64)
    y = np.ascontiguousarray(mesh.y, dtype=np.float64)
    ien = np.ascontiguousarray(mesh.ien, dtype=np.int32).reshape(-1)
    zz = None if z is None else np.ascontiguousarray(z, dtype=np.float64)
    check(lib().fg_write_vtu(os.fsencode(path), mesh.nnodes, mesh.nel, x.ctypes.data, y.ctypes.data, ien.ctypes.data,
                             len(fields), ctypes.addressof(arr), None if zz is None else zz.ctypes.data))


def node_values(mesh, u, upresc):
    """Per-node dof values (nnodes x ndof, squeezed for ndof = 1): free dofs
    from the solution u (invP_id numbering), prescribed ones from upresc, as
    every Paraview_Output.c gathers them before writing."""
    u = np.asarray(u, dtype=np.float64)
    up = np.asarray(upresc, dtype=np.float64).reshape(-1)
    v = np.where(mesh.type > 0, u[np.maximum(mesh.invp, 0)], up)
    return v if mesh.ndof == 1 else v.reshape(mesh.nnodes, mesh.ndof)


def write_transport_vtu(path, prob, u):
    """SST / transient transport output: "solucao" with points lifted by u."""
    v = node_values(prob.mesh, u, prob.upresc)
    write_vtu(path, prob.mesh, {"solucao": v}, z=v)


def write_euler_vtu(path, prob, U, cv=716.5):
    """Euler output: Density, Temperature, Pressure from the conserved
    variables (rho, rho u, rho v, rho E); cv is the problem's cv(x, y)."""
    V = node_values(prob.mesh, U, prob.upresc)
    rho, m1, m2, e = V[:, 0], V[:, 1], V[:, 2], V[:, 3]
    aux = e - (m1 * m1 + m2 * m2) / (2.0 * rho)
    write_vtu(path, prob.mesh, {"Density": rho, "Temperature": aux / (rho * cv), "Pressure": (prob.gamma - 1) * aux})


def write_ns_vtu(path, prob, U):
    """Navier-Stokes output: Velocity (u, v, 0) and Pressure."""
    V = node_values(prob.mesh, U, prob.upresc)
    write_vtu(path, prob.mesh, {"Velocity": V[:, :2], "Pressure": V[:, 2]})


def mesh_analyze(mesh, reorder: bool = True) -> dict:
    """Host-only set-up products (no GPU): lm, Perm, invPerm, colour, info."""
    S = 3 * mesh.ndof
    lm = np.empty(mesh.nel * S, dtype=np.int32)
    perm = np.empty(mesh.neq + 1, dtype=np.int32)
    inv = np.empty(mesh.neq + 1, dtype=np.int32)
    col = np.empty(max(mesh.nel, 1), dtype=np.int32)
    info = SystemInfo()
    check(lib().fg_mesh_analyze(mesh.nnodes, mesh.nel, mesh.ndof,
                                np.ascontiguousarray(mesh.ien, dtype=np.int32).reshape(-1),
                                np.ascontiguousarray(mesh.type, dtype=np.int32),
                                np.ascontiguousarray(mesh.invp, dtype=np.int32), mesh.neq,
                                FG_REORDER_RCM if reorder else FG_REORDER_NONE,
                                lm.ctypes.data, perm.ctypes.data, inv.ctypes.data, col.ctypes.data,
                                ctypes.byref(info)))
    return {"lm": lm.reshape(mesh.nel, S), "perm": perm, "invperm": inv, "colour": col[:mesh.nel],
            "info": {k: getattr(info, k) for k, _ in info._fields_}}


@dataclasses.dataclass
class SolveResult:
    x: np.ndarray
    stats: dict


class System:
    """One EBE linear system on the GPU: mesh connectivity, element blocks,
    preconditioner and resident solver state."""

    def __init__(self, mesh, reorder: bool = True):
        self.mesh = mesh
        h = _vp()
        check(lib().fg_system_create(ctypes.byref(h), mesh.nnodes, mesh.nel, mesh.ndof,
                                     np.ascontiguousarray(mesh.ien, dtype=np.int32).reshape(-1),
                                     np.ascontiguousarray(mesh.type, dtype=np.int32),
                                     np.ascontiguousarray(mesh.invp, dtype=np.int32), mesh.neq,
                                     FG_REORDER_RCM if reorder else FG_REORDER_NONE))
        self._h = h
        self.n = mesh.neq
        self.S = 3 * mesh.ndof

    def close(self):
        if getattr(self, "_h", None):
            lib().fg_system_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        """cudaStream_t of this system's work, as an integer handle."""
        return int(lib().fg_system_stream(self._h) or 0)

    def info(self) -> dict:
        i = SystemInfo()
        check(lib().fg_system_get_info(self._h, ctypes.byref(i)))
        return {k: getattr(i, k) for k, _ in i._fields_}

    def lm(self):
        out = np.empty(self.mesh.nel * self.S, dtype=np.int32)
        check(lib().fg_system_get_lm(self._h, out))
        return out.reshape(self.mesh.nel, self.S)

    def perm(self):
        p = np.empty(self.n + 1, dtype=np.int32)
        q = np.empty(self.n + 1, dtype=np.int32)
        check(lib().fg_system_get_perm(self._h, p, q))
        return p, q

    def colours(self):
        c = np.empty(self.mesh.nel, dtype=np.int32)
        check(lib().fg_system_get_colours(self._h, c))
        return c

    def set_operator(self, op):
        check(lib().fg_set_operator(self._h, op))

    def set_spike(self, k=16, parts=16):
        """Coupling size and block count of the SPIKE preconditioner."""
        check(lib().fg_set_spike(self._h, int(k), int(parts)))

    def set_ilu_blocks(self, blocks):
        """Block-Jacobi ILU over `blocks` row blocks (1: global ILU)."""
        check(lib().fg_set_ilu_blocks(self._h, int(blocks)))

    def set_ilu_fill(self, p):
        """Fill level of FG_PRECOND_ILU0 (Preconditioner "ILU<p>")."""
        check(lib().fg_set_ilu_fill(self._h, int(p)))

    def csr(self):
        """(IA, JA, AA) of the assembled operator in the internal (RCM) numbering."""
        nnz = _c_int(0)
        check(lib().fg_get_csr(self._h, ctypes.byref(nnz), None, None, None))
        IA = np.empty(self.n + 1, dtype=np.int32)
        JA = np.empty(max(nnz.value, 1), dtype=np.int32)
        AA = np.empty(max(nnz.value, 1))
        check(lib().fg_get_csr(self._h, None, IA.ctypes.data, JA.ctypes.data, AA.ctypes.data))
        return IA, JA[:nnz.value], AA[:nnz.value]

    def set_blocks(self, A):
        check(lib().fg_set_blocks(self._h, np.ascontiguousarray(A, dtype=np.float64).reshape(-1)))

    def get_blocks(self):
        A = np.empty(self.mesh.nel * self.S * self.S)
        check(lib().fg_get_blocks(self._h, A))
        return A.reshape(self.mesh.nel, self.S * self.S)

    def matvec(self, P, precision=64):
        P = np.ascontiguousarray(P, dtype=np.float64)
        Q = np.empty(self.n + 1)
        check(lib().fg_matvec(self._h, P, Q, precision))
        return Q

    def precond_setup(self, kind=FG_PRECOND_DIAG, flags=0, F=None):
        Fc = None if F is None else np.array(F, dtype=np.float64, copy=True)
        check(lib().fg_precond_setup(self._h, kind, flags, _ptr(Fc)))
        return Fc

    def scale(self, kind, F=None):
        """Left or left-right diagonal scaling of the blocks; returns scaled F."""
        Fc = None if F is None else np.array(F, dtype=np.float64, copy=True)
        check(lib().fg_scale(self._h, kind, _ptr(Fc)))
        return Fc

    def unscale(self, X):
        Xc = np.array(X, dtype=np.float64, copy=True)
        check(lib().fg_unscale(self._h, Xc.ctypes.data))
        return Xc

    def precond_apply(self, p):
        p = np.ascontiguousarray(p, dtype=np.float64)
        z = np.empty(self.n + 1)
        check(lib().fg_precond_apply(self._h, p, z))
        return z

    def precond_apply_right(self, p):
        """The right preconditioner of the set-up (SGSe's backward sweep; the
        identity for the other kinds)."""
        p = np.ascontiguousarray(p, dtype=np.float64)
        z = np.empty(self.n + 1)
        check(lib().fg_precond_apply_right(self._h, p, z))
        return z

    def diag(self):
        d = np.empty(self.n + 1)
        check(lib().fg_get_diag(self._h, d))
        return d

    def solve(self, B, kmax=30, lmax=1000, tol=1e-10, precision=FG_PREC_FP64, inner_tol=0.0, F_true=None):
        B = np.ascontiguousarray(B, dtype=np.float64)
        X = np.zeros(self.n + 1)
        o = SolverOpts(kmax, lmax, tol, precision, inner_tol)
        st = SolveStats()
        Ft = None if F_true is None else np.ascontiguousarray(F_true, dtype=np.float64)
        check(lib().fg_solve(self._h, ctypes.byref(o), B, X, _ptr(Ft), ctypes.byref(st)))
        return SolveResult(X, st.as_dict())

    # ---- transport assembly
    def set_geometry(self, x, y, upresc):
        check(lib().fg_set_geometry(self._h, np.ascontiguousarray(x, dtype=np.float64),
                                    np.ascontiguousarray(y, dtype=np.float64),
                                    np.ascontiguousarray(upresc, dtype=np.float64)))

    def transport_assemble(self, prob, u=None):
        c = _coeffs(prob)
        F = np.empty(self.n + 1)
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        check(lib().fg_transport_assemble(self._h, ctypes.byref(c), _ptr(uu), F.ctypes.data))
        return F

    def transport_prepare(self, prob, u=None):
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        check(lib().fg_transport_prepare(self._h, ctypes.byref(_coeffs(prob)), _ptr(uu)))

    def solution(self):
        X = np.empty(self.n + 1)
        check(lib().fg_get_solution(self._h, X))
        return X

    def transport_process(self, prob, kmax=30, lmax=1000, tol=1e-10, nonlinear_tol=1e-3, max_nonlinear=1000,
                          precision=FG_PREC_FP64):
        c = _coeffs(prob)
        o = SolverOpts(kmax, lmax, tol, precision, 0.0)
        U = np.zeros(self.n)
        st = ProcessStats()
        check(lib().fg_transport_process(self._h, ctypes.byref(c), ctypes.byref(o), nonlinear_tol, max_nonlinear,
                                         U, ctypes.byref(st)))
        return U, {k: getattr(st, k) for k, _ in st._fields_}

    # ---- steady Navier-Stokes (ndof = 3)
    def ns_set_geometry(self, prob):
        f1 = np.ascontiguousarray(prob.f1, dtype=np.float64)
        f2 = np.ascontiguousarray(prob.f2, dtype=np.float64)
        check(lib().fg_ns_set_geometry(self._h, np.ascontiguousarray(self.mesh.x, dtype=np.float64),
                                       np.ascontiguousarray(self.mesh.y, dtype=np.float64),
                                       np.ascontiguousarray(prob.upresc, dtype=np.float64),
                                       f1.ctypes.data, f2.ctypes.data))

    def ns_assemble(self, prob, u=None, form=FG_NS_SUPG_PSPG):
        """Build_K_F_SUPG_PSPG (or Build_K_F_VMS_DCDD with form=FG_NS_VMS_DCDD)
        at u (free dofs, reference numbering); returns F (n+1)."""
        c = NSCoeffs(prob.reynolds, FG_PRECOND_BLOCKDIAG, form)
        F = np.empty(self.n + 1)
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        check(lib().fg_ns_assemble(self._h, ctypes.byref(c), _ptr(uu), F.ctypes.data))
        return F

    def ns_process(self, prob, u0=None, kmax=30, lmax=1000, tol=1e-10, nonlinear_tol=1e-3, max_nonlinear=100,
                   precision=FG_PREC_FP64, inner_tol=0.0, precond=FG_PRECOND_BLOCKDIAG, form=FG_NS_SUPG_PSPG):
        """Picard loop from u0 (default 0); returns (u[n], stats)."""
        c = NSCoeffs(prob.reynolds, precond, form)
        o = SolverOpts(kmax, lmax, tol, precision, inner_tol)
        u = np.zeros(self.n) if u0 is None else np.array(u0, dtype=np.float64, copy=True)
        st = ProcessStats()
        check(lib().fg_ns_process(self._h, ctypes.byref(c), ctypes.byref(o), nonlinear_tol, max_nonlinear, u,
                                  ctypes.byref(st)))
        return u, {k: getattr(st, k) for k, _ in st._fields_}

    # ---- transient transport (ndof = 1, geometry from set_geometry)
    def tt_assemble(self, prob, alpha, dt, u=None, du=None):
        """Build_M_K_R_SUPG at (u, du); returns R (n+1); blocks stay on the device."""
        c = tt_coeffs(prob, alpha, dt)
        R = np.empty(self.n + 1)
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        dd = None if du is None else np.ascontiguousarray(du, dtype=np.float64)
        check(lib().fg_tt_assemble(self._h, ctypes.byref(c), _ptr(uu), _ptr(dd), R.ctypes.data))
        return R

    def tt_bubble_assemble(self, prob, alpha, dt, u=None, du=None, uB=None, duB=None):
        """Build_M_F_DD ("Predictor2", form DD) at (u, du) and the bubble
        unknowns (uB, duB: one per element, reference order) with a fresh
        shock-capture state; returns (F[n+1], cond[nel, 5] = invN2, R2,
        M2[0..2]); the blocks stay on the device."""
        c = tt_coeffs(prob, alpha, dt)
        nel = self.mesh.nel
        F = np.empty(self.n + 1)
        cond = np.empty(5 * max(nel, 1))
        arr = [None if v is None else np.ascontiguousarray(v, dtype=np.float64) for v in (u, du, uB, duB)]
        check(lib().fg_tt_bubble_assemble(self._h, ctypes.byref(c), *[_ptr(v) for v in arr], F.ctypes.data,
                                          cond.ctypes.data))
        return F, cond[: 5 * nel].reshape(nel, 5)

    def _bubble_nb(self):
        return 4 if self.S == 12 else 1

    def bubble_dab(self, Da):
        """calculate_DaB after the last Predictor2 build: DaB (1 or 4 per
        element, element-major) from Da (n+1)."""
        Da = np.ascontiguousarray(Da, dtype=np.float64)
        if Da.shape != (self.n + 1,):
            raise ValueError("Da needs n + 1 entries")
        m = self._bubble_nb() * self.mesh.nel
        DaB = np.empty(max(m, 1))
        check(lib().fg_bubble_dab(self._h, Da.ctypes.data, DaB.ctypes.data))
        return DaB[:m]

    def bubble_state(self):
        """(uB, aB) after a Predictor2 loop (FG_TIME_PREDICTOR2)."""
        m = self._bubble_nb() * self.mesh.nel
        uB, aB = np.empty(max(m, 1)), np.empty(max(m, 1))
        check(lib().fg_bubble_state(self._h, uB.ctypes.data, aB.ctypes.data))
        return uB[:m], aB[:m]

    def euler_bubble_assemble(self, prob, u=None, du=None, uB=None, duB=None):
        """Build_M_F_DD_Transiente (Euler "Predictor2", DD, YZBeta) at (u, du)
        and the bubble unknowns (4 per element) with fresh shock-capture
        states; returns (F[n+1], cond[nel, 53] = invN2, R2[4], M2[4][12]);
        the blocks stay on the device."""
        c = euler_coeffs(prob)
        nel = self.mesh.nel
        F = np.empty(self.n + 1)
        cond = np.empty(53 * max(nel, 1))
        arr = [None if v is None else np.ascontiguousarray(v, dtype=np.float64) for v in (u, du, uB, duB)]
        check(lib().fg_euler_bubble_assemble(self._h, ctypes.byref(c), *[_ptr(v) for v in arr], F.ctypes.data,
                                             cond.ctypes.data))
        return F, cond[: 53 * nel].reshape(nel, 53)

    def tt_predictor(self, prob, alpha, dt, topts, u0=None, kmax=30, lmax=1000, tol=1e-10,
                     precision=FG_PREC_FP64, inner_tol=0.0):
        """Predictor_Old with the transient transport build; returns (u, a, stats)."""
        c = tt_coeffs(prob, alpha, dt)
        o = SolverOpts(kmax, lmax, tol, precision, inner_tol)
        u = np.zeros(self.n) if u0 is None else np.array(u0, dtype=np.float64, copy=True)
        u = np.ascontiguousarray(u, dtype=np.float64)
        a = np.zeros(self.n)
        st = TimeStats()
        check(lib().fg_tt_predictor(self._h, ctypes.byref(c), ctypes.byref(o), ctypes.byref(topts), u,
                                    a.ctypes.data, ctypes.byref(st)))
        return u, a, {k: getattr(st, k) for k, _ in st._fields_}

    # ---- compressible Euler (ndof = 4)
    def euler_set_geometry(self, prob):
        check(lib().fg_euler_set_geometry(self._h, np.ascontiguousarray(self.mesh.x, dtype=np.float64),
                                          np.ascontiguousarray(self.mesh.y, dtype=np.float64),
                                          np.ascontiguousarray(prob.upresc, dtype=np.float64)))

    def euler_assemble(self, prob, u=None, du=None):
        """Build_M_K_F_SUPG at (u, du) (free dofs, reference numbering); returns R (n+1)."""
        c = euler_coeffs(prob)
        R = np.empty(self.n + 1)
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        dd = None if du is None else np.ascontiguousarray(du, dtype=np.float64)
        check(lib().fg_euler_assemble(self._h, ctypes.byref(c), _ptr(uu), _ptr(dd), R.ctypes.data))
        return R

    def euler_predictor(self, prob, topts, u0=None, kmax=25, lmax=1000, tol=1e-10, precision=FG_PREC_FP64,
                        inner_tol=0.0):
        """Predictor_Old from u0 (default: the problem's initial state); returns (u, a, stats)."""
        c = euler_coeffs(prob)
        o = SolverOpts(kmax, lmax, tol, precision, inner_tol)
        u = prob.initial_state() if u0 is None else np.array(u0, dtype=np.float64, copy=True)
        u = np.ascontiguousarray(u, dtype=np.float64)
        a = np.zeros(self.n)
        st = TimeStats()
        check(lib().fg_euler_predictor(self._h, ctypes.byref(c), ctypes.byref(o), ctypes.byref(topts), u,
                                       a.ctypes.data, ctypes.byref(st)))
        return u, a, {k: getattr(st, k) for k, _ in st._fields_}


def tt_coeffs(prob, alpha, dt) -> TTCoeffs:
    """Transient transport coefficients of a transport problem."""
    return TTCoeffs(_coeffs(prob), float(alpha), float(dt))


def euler_coeffs(prob) -> EulerCoeffs:
    """Euler coefficients of a problem; invY (the YZBeta scaling of
    "Predictor2") from prob.invY, default ones."""
    iy = [float(v) for v in getattr(prob, "invY", (1.0, 1.0, 1.0, 1.0))]
    return EulerCoeffs(prob.gamma, prob.mach, int(prob.dimensionless), prob.tolerance, prob.alpha, prob.dt,
                       int(getattr(prob, "form", 0)), (_c_dbl * 4)(*iy), int(getattr(prob, "shock", 0)))


def time_opts(stop_by_norm=0, max_corrections=2, correction_tol=1e-3, steady_state=0, final_time=0.0,
              time_tol=1e-6, max_steps=0, precond=None, setup_flags=None, scheme=0) -> TimeOpts:
    """Criteria.c controls and the TimeIntegration scheme (FG_TIME_*); the
    preconditioner defaults to the reference's BlockDiag with its 4x4
    inverse (FG_SETUP_REF_QUIRKS)."""
    precond = FG_PRECOND_BLOCKDIAG if precond is None else precond
    setup_flags = FG_SETUP_REF_QUIRKS if setup_flags is None else setup_flags
    return TimeOpts(stop_by_norm, max_corrections, correction_tol, steady_state, final_time, time_tol, max_steps,
                    precond, setup_flags, scheme)


def euler_system(prob, reorder=False) -> System:
    """A System (ndof = 4; node-order numbering, or RCM with reorder=True,
    as the CSR/ILU(0) configuration uses) with the geometry and prescribed
    values of an Euler problem."""
    s = System(prob.mesh, reorder=reorder)
    s.euler_set_geometry(prob)
    return s


def ns_system(prob, reorder=False) -> System:
    """A System (ndof = 3; node-order numbering, or RCM with reorder=True)
    with the geometry, prescribed values and body force of a Navier-Stokes
    problem."""
    s = System(prob.mesh, reorder=reorder)
    s.ns_set_geometry(prob)
    return s


def _coeffs(prob):
    return TransportCoeffs(prob.k, prob.gamma, (_c_dbl * 2)(*prob.beta), prob.f, int(prob.cau),
                           int(getattr(prob, "form", 0)), int(getattr(prob, "h_shock", 0)))


def set_wait_limit(polls=1 << 24):
    """Polls of the ILU kernels' bounded dependency waits (current device)."""
    check(lib().fg_set_wait_limit(ctypes.c_longlong(int(polls))))


def set_memory_limit(nbytes=0):
    """Cap on the device bytes the library allocates (0: none)."""
    check(lib().fg_set_memory_limit(int(nbytes)))


def memory_in_use() -> int:
    return int(lib().fg_memory_in_use())


def launch_count() -> int:
    return int(lib().fg_launch_count())


def solve_batch(systems, Bs, F_trues=None, kmax=30, lmax=1000, tol=1e-10, precision=FG_PREC_FP64, inner_tol=0.0):
    """Solve systems together (host vectors); returns (list of X, list of stats)."""
    n = len(systems)
    H = (_vp * n)(*[s.handle for s in systems])
    Bs = [np.ascontiguousarray(b, dtype=np.float64) for b in Bs]
    Xs = [np.zeros(s.n + 1) for s in systems]
    Bp = (_vp * n)(*[b.ctypes.data for b in Bs])
    Xp = (_vp * n)(*[x.ctypes.data for x in Xs])
    Fp = None
    if F_trues is not None:
        F_trues = [np.ascontiguousarray(f, dtype=np.float64) for f in F_trues]
        Fp = (_vp * n)(*[f.ctypes.data for f in F_trues])
    st = (SolveStats * n)()
    o = SolverOpts(kmax, lmax, tol, precision, inner_tol)
    check(lib().fg_solve_batch(ctypes.cast(H, _vp), n, ctypes.byref(o), ctypes.cast(Bp, _vp), ctypes.cast(Xp, _vp),
                               None if Fp is None else ctypes.cast(Fp, _vp), ctypes.cast(st, _vp)))
    return Xs, [s.as_dict() for s in st]


def autotune(systems, kmax=30, lmax=1000, tol=1e-10, precision=FG_PREC_MIXED, inner_tol=0.0, remeasure=False):
    """Time candidate launch shapes on this batch (resident right-hand sides
    required) and keep the fastest for its key; returns the choice."""
    n = len(systems)
    H = (_vp * n)(*[s.handle for s in systems])
    o = SolverOpts(kmax, lmax, tol, precision, inner_tol)
    c = TuneChoice()
    check(lib().fg_autotune(ctypes.cast(H, _vp), n, ctypes.byref(o), int(bool(remeasure)), ctypes.byref(c)))
    return c.as_dict()


def tune_lookup(systems, kmax=30, lmax=1000, tol=1e-10, precision=FG_PREC_MIXED, inner_tol=0.0):
    n = len(systems)
    H = (_vp * n)(*[s.handle for s in systems])
    o = SolverOpts(kmax, lmax, tol, precision, inner_tol)
    c = TuneChoice()
    check(lib().fg_tune_lookup(ctypes.cast(H, _vp), n, ctypes.byref(o), ctypes.byref(c)))
    return c.as_dict()


def tune_set(systems, part_dofs, mv3_pipeline=1, kmax=30, lmax=1000, tol=1e-10, precision=FG_PREC_MIXED,
             inner_tol=0.0):
    """Install a launch-shape choice for this batch's key without timing."""
    n = len(systems)
    H = (_vp * n)(*[s.handle for s in systems])
    o = SolverOpts(kmax, lmax, tol, precision, inner_tol)
    c = TuneChoice(part_dofs, mv3_pipeline, 0.0, 0, 0)
    check(lib().fg_tune_set(ctypes.cast(H, _vp), n, ctypes.byref(o), ctypes.byref(c)))


def tune_clear():
    lib().fg_tune_clear()


def solve_resident(systems, kmax=30, lmax=1000, tol=1e-10, precision=FG_PREC_FP64, inner_tol=0.0):
    """Solve systems with their device-resident right-hand sides; returns stats."""
    n = len(systems)
    H = (_vp * n)(*[s.handle for s in systems])
    st = (SolveStats * n)()
    o = SolverOpts(kmax, lmax, tol, precision, inner_tol)
    check(lib().fg_solve_resident(ctypes.cast(H, _vp), n, ctypes.byref(o), ctypes.cast(st, _vp)))
    return [s.as_dict() for s in st]


def bench_matvec(systems, precision=32, reps=20):
    """(ms per batched matvec, algorithmic bytes per matvec) timed with CUDA events."""
    n = len(systems)
    H = (_vp * n)(*[s.handle for s in systems])
    ms, b = _c_dbl(), _c_dbl()
    check(lib().fg_bench_matvec(ctypes.cast(H, _vp), n, precision, reps, ctypes.byref(ms), ctypes.byref(b)))
    return ms.value, b.value


class Server:
    """Continuous-batching request server (fg_server_*): submit transport
    requests and Euler time loops at any time, poll finished results with
    their timestamps (Euler results carry the final state as "u")."""

    def __init__(self, kmax=30, lmax=10000, tol=1e-10, precision=FG_PREC_MIXED, inner_tol=0.0,
                 hbm_budget_bytes=0, max_active=0):
        h = _vp()
        o = ServerOpts(kmax, lmax, tol, precision, inner_tol, hbm_budget_bytes, max_active)
        check(lib().fg_server_create(ctypes.byref(h), ctypes.byref(o)))
        self._h = h
        self._keep = {}

    def submit(self, system, prob, tag):
        c = _coeffs(prob)
        self._keep[tag] = system
        check(lib().fg_server_submit(self._h, system.handle, ctypes.byref(c), tag))

    def submit_host(self, system, A, F, X, tag):
        """A request with host buffers: blocks A (nel x S*S), right-hand side
        F (n+1); X (n+1, float64, C-contiguous) receives the solution before
        the result is polled.  The arrays are kept alive until then."""
        if not (isinstance(X, np.ndarray) and X.dtype == np.float64 and X.flags.c_contiguous):
            raise ValueError("X must be a C-contiguous float64 array")
        A = np.ascontiguousarray(A, dtype=np.float64)
        F = np.ascontiguousarray(F, dtype=np.float64)
        self._keep[tag] = (system, A, F, X)
        check(lib().fg_server_submit_host(self._h, system.handle, A.reshape(-1), F, X, tag))

    def submit_euler(self, system, prob, topts, tag, u0=None):
        c = euler_coeffs(prob)
        u = prob.initial_state() if u0 is None else np.array(u0, dtype=np.float64, copy=True)
        u = np.ascontiguousarray(u, dtype=np.float64)
        self._keep[tag] = (system, u, topts)
        check(lib().fg_server_submit_euler(self._h, system.handle, ctypes.byref(c), ctypes.byref(topts), u, tag))

    def now(self) -> float:
        return float(lib().fg_server_now(self._h))

    def wait(self, n, timeout=60.0):
        check(lib().fg_server_wait(self._h, n, timeout))

    def poll(self, max_results=4096):
        buf = (ServerResult * max_results)()
        cnt = _c_int(0)
        check(lib().fg_server_poll(self._h, ctypes.cast(buf, _vp), max_results, ctypes.byref(cnt)))
        out = [buf[i].as_dict() for i in range(cnt.value)]
        for r in out:
            kept = self._keep.pop(r["tag"], None)
            if isinstance(kept, tuple):
                r["u"] = kept[1]
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().fg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def transport_system(prob, reorder=True) -> System:
    """A System with the geometry and Dirichlet data of a transport problem."""
    s = System(prob.mesh, reorder=reorder)
    s.set_geometry(prob.mesh.x, prob.mesh.y, prob.upresc)
    return s
