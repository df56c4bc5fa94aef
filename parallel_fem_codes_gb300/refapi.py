"""The reference's steady-transport structs and entry points, from Python.

`libfemgpu_sst.so` exports the reference's solve-path functions (pgmres,
ebemv, Diag_precond, Diag_precond_EBE_setup, NO_precond, NO_precond_setup)
with the reference's signatures, running on the GPU.  This module mirrors
the structs those functions take (SSTranspEquation.h:17-163, restated in
compat/femgpu_ref_sst.h) and builds the state the reference's Preprocess.c
leaves behind for one rank, so a driver written against the reference's
interface can be exercised from Python (the tests do).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import build as _build

c_int, c_dbl, c_char = ctypes.c_int, ctypes.c_double, ctypes.c_char
P_dbl, P_int = ctypes.POINTER(c_dbl), ctypes.POINTER(c_int)


class NodeType(ctypes.Structure):
    _fields_ = [("x", c_dbl), ("y", c_dbl), ("Type", c_int), ("Send", c_int), ("invP_id", c_int)]


class ElementType(ctypes.Structure):
    _fields_ = [("Vertex", c_int * 3), ("Type", c_int)]


class ParametersType(ctypes.Structure):
    _fields_ = [(n, c_char * 200) for n in ("ProblemTitle", "Solver", "Preconditioner", "Scaling", "reordering",
                                            "MatrixVectorProductScheme", "StabilizationForm", "ShockCapture",
                                            "h_Shock")] + \
               [("SolverTolerance", c_dbl), ("NonLinearTolerance", c_dbl)] + \
               [(n, c_int) for n in ("KrylovBasisVectorsQuantity", "nnodes", "nNodes", "nel", "nEl", "neq",
                                     "neq_bef", "neqaux_bef", "neqaux_aft", "nsend_bef", "nsend_aft", "nrecv_bef",
                                     "nrecv_aft", "NEQ", "nedge", "nnzero", "nnzero_bef", "nnzero_aft",
                                     "LinearMaxIter", "iterations", "k_SPIKE_block_size", "bandwidth_bef",
                                     "bandwidth_aft", "RANK", "NPROC")] + \
               [("arguments", ctypes.c_void_p), ("PardisoVariables", ctypes.c_void_p)]


class MatrixDataType(ctypes.Structure):
    _fields_ = [("A", ctypes.POINTER(P_dbl)), ("Aaux", P_dbl), ("AA", P_dbl), ("AA_bef", P_dbl), ("AA_aft", P_dbl),
                ("Diag", P_dbl), ("invDiag", P_dbl)] + \
               [(n, ctypes.c_void_p) for n in ("Scheme_by_Element", "Scheme_by_Element_bef", "Scheme_by_Element_aft",
                                               "order", "JA", "IA", "JA_bef", "IA_bef", "JA_aft", "IA_aft", "aux_bef",
                                               "aux_aft", "ILUp", "mat", "Ailu")] + \
               [("Perm", P_int), ("invPerm", P_int)] + \
               [(n, ctypes.c_void_p) for n in ("fullC", "fullCaux", "fullB", "fullBaux", "LUe", "LUeaux",
                                               "A_SPIKE", "B_SPIKE", "C_SPIKE", "S_SPIKE")]


class FemStructsType(ctypes.Structure):
    _fields_ = [("lm", ctypes.POINTER(P_int)), ("lmaux", P_int), ("Node", ctypes.POINTER(NodeType)),
                ("Element", ctypes.POINTER(ElementType))] + \
               [(n, P_dbl) for n in ("delta_old", "Re_old", "F", "U", "u", "f", "SendBuffer_bef", "SendBuffer_aft",
                                     "RecvBuffer_bef", "RecvBuffer_aft")] + \
               [(n, P_int) for n in ("IdSend_bef", "IdSend_aft", "IdRecv_bef", "IdRecv_aft")]


FN = ctypes.CFUNCTYPE(c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)


class FemFunctionsType(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("Condutivity", "Font", "Reaction", "Velocity", "upresc",
                                               "h_shock_calculation", "ShockCapture", "assembly", "mv", "precond",
                                               "precondR", "precond_setup", "scaling", "unscaling")]


def layout_offsets():
    """The same 37 numbers fgc_sst_layout / the reference harness report."""
    P, M, S, F = ParametersType, MatrixDataType, FemStructsType, FemFunctionsType
    return [ctypes.sizeof(P), P.SolverTolerance.offset, P.KrylovBasisVectorsQuantity.offset, P.nnodes.offset,
            P.nel.offset, P.neq.offset, P.neq_bef.offset, P.NEQ.offset, P.LinearMaxIter.offset, P.iterations.offset,
            P.RANK.offset, P.NPROC.offset, ctypes.sizeof(M), M.A.offset, M.Aaux.offset, M.Diag.offset,
            M.invDiag.offset, M.Perm.offset, M.invPerm.offset, ctypes.sizeof(S), S.lm.offset, S.lmaux.offset,
            S.Node.offset, S.Element.offset, ctypes.sizeof(F), F.mv.offset, F.precond.offset, F.precondR.offset,
            F.precond_setup.offset, ctypes.sizeof(NodeType), ctypes.sizeof(ElementType), M.AA.offset, M.JA.offset,
            M.IA.offset, P.MatrixVectorProductScheme.offset, P.Preconditioner.offset, P.nnzero.offset]


_shim = None


def shim():
    """libfemgpu_sst.so (built with the package)."""
    global _shim
    if _shim is None:
        _build.build()
        L = ctypes.CDLL(_build.COMPAT_SST)
        for name in ("pgmres",):
            getattr(L, name).argtypes = [ctypes.c_void_p] * 6
        for name in ("ebemv", "Diag_precond", "NO_precond"):
            getattr(L, name).argtypes = [ctypes.c_void_p] * 5
        for name in ("Diag_precond_EBE_setup", "NO_precond_setup"):
            getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_int, ctypes.c_void_p]
        L.fgc_sst_layout.argtypes = [np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")]
        L.fgc_sst_layout.restype = None
        _shim = L
    return _shim


def _addr(lib, name):
    return ctypes.cast(getattr(lib, name), ctypes.c_void_p).value


class DriverState:
    """The structs Preprocess.c fills for one rank (EBE storage, Diag
    preconditioning, GMRES), holding numpy arrays the driver owns."""

    def __init__(self, mesh, kmax=30, lmax=1000, tol=1e-10, precond="Diag"):
        L = shim()
        n, nel, nn = mesh.neq, mesh.nel, mesh.nnodes
        self.P = ParametersType()
        for k, v in (("Solver", b"GMRES"), ("Preconditioner", precond.encode()), ("Scaling", b"NOT"),
                     ("reordering", b"SYMRCM"), ("MatrixVectorProductScheme", b"EBE")):
            setattr(self.P, k, v)
        self.P.SolverTolerance, self.P.KrylovBasisVectorsQuantity, self.P.LinearMaxIter = tol, kmax, lmax
        self.P.nnodes = self.P.nNodes = nn
        self.P.nel = self.P.nEl = nel
        self.P.neq = self.P.NEQ = n
        self.P.NPROC = 1
        self.nodes = (NodeType * nn)()
        for i in range(nn):
            t = int(mesh.type[i])
            self.nodes[i].x, self.nodes[i].y = float(mesh.x[i]), float(mesh.y[i])
            self.nodes[i].Type, self.nodes[i].Send = t, 1
            self.nodes[i].invP_id = int(mesh.invp[i]) if t else -1
        self.elems = (ElementType * nel)()
        for e in range(nel):
            for v in range(3):
                self.elems[e].Vertex[v] = int(mesh.ien[e, v])
        self.Aaux = np.zeros(nel * 9)
        self.rows = (P_dbl * nel)(*[ctypes.cast(self.Aaux.ctypes.data + 72 * e, P_dbl) for e in range(nel)])
        self.Diag = np.zeros(n + 1)
        self.invDiag = np.zeros(n + 1)
        self.M = MatrixDataType()
        self.M.A = ctypes.cast(self.rows, ctypes.POINTER(P_dbl))
        self.M.Aaux = self.Aaux.ctypes.data_as(P_dbl)
        self.M.Diag = self.Diag.ctypes.data_as(P_dbl)
        self.M.invDiag = self.invDiag.ctypes.data_as(P_dbl)
        self.S = FemStructsType()
        self.S.Node = ctypes.cast(self.nodes, ctypes.POINTER(NodeType))
        self.S.Element = ctypes.cast(self.elems, ctypes.POINTER(ElementType))
        self.Fn = FemFunctionsType()
        self.Fn.mv = _addr(L, "ebemv")
        self.Fn.precond = _addr(L, "Diag_precond" if precond == "Diag" else "NO_precond")
        self.Fn.precondR = _addr(L, "NO_precond")
        self.setup = getattr(L, "Diag_precond_EBE_setup" if precond == "Diag" else "NO_precond_setup")

    def ptrs(self):
        return (ctypes.addressof(self.P), ctypes.addressof(self.M), ctypes.addressof(self.S))

    def precond_setup(self, F):
        F = np.array(F, dtype=np.float64, copy=True)
        rc = self.setup(*self.ptrs(), 1, F.ctypes.data)
        return rc, F

    def pgmres(self, B):
        B = np.ascontiguousarray(B, dtype=np.float64)
        X = np.zeros_like(B)
        rc = shim().pgmres(*self.ptrs(), ctypes.addressof(self.Fn), B.ctypes.data, X.ctypes.data)
        return rc, X

    def ebemv(self, P):
        Pv = np.array(P, dtype=np.float64, copy=True)
        Q = np.zeros_like(Pv)
        rc = shim().ebemv(*self.ptrs(), Pv.ctypes.data, Q.ctypes.data)
        return rc, Q
