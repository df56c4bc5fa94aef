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

from parallel_fem_codes_gb300 import build as _build

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
        for name in ("ebemv", "Diag_precond", "NO_precond", "csrmv", "ILUp_precond", "SPIKE_precond"):
            getattr(L, name).argtypes = [ctypes.c_void_p] * 5
        L.csr_assembly.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_int, ctypes.c_void_p]
        L.csr_assembly.restype = None
        for name in ("Diag_precond_EBE_setup", "NO_precond_setup", "ILUp_precond_setup", "SPIKE_precond_setup"):
            getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_int, ctypes.c_void_p]
        L.fgc_sst_layout.argtypes = [np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")]
        L.fgc_sst_layout.restype = None
        _shim = L
    return _shim


def _addr(lib, name):
    return ctypes.cast(getattr(lib, name), ctypes.c_void_p).value


class DriverState:
    """The structs Preprocess.c fills for one rank (EBE or CSR storage;
    Diag, ILU0, SPIKEk or no preconditioning; GMRES), holding numpy arrays
    the driver owns."""

    def __init__(self, mesh, kmax=30, lmax=1000, tol=1e-10, precond="Diag", scheme="EBE"):
        L = shim()
        n, nel, nn = mesh.neq, mesh.nel, mesh.nnodes
        self.P = ParametersType()
        for k, v in (("Solver", b"GMRES"), ("Preconditioner", precond.encode()), ("Scaling", b"NOT"),
                     ("reordering", b"SYMRCM"), ("MatrixVectorProductScheme", scheme.encode())):
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
        kind = "Diag" if precond == "Diag" else "ILUp" if precond.startswith("ILU") else \
            "SPIKE" if precond.startswith("SPIKE") else "NO"
        self.Fn.mv = _addr(L, "csrmv" if scheme == "CSR" else "ebemv")
        self.Fn.assembly = _addr(L, "csr_assembly") if scheme == "CSR" else None
        self.Fn.precond = _addr(L, kind + "_precond")
        self.Fn.precondR = _addr(L, "NO_precond")
        self.setup = getattr(L, {"Diag": "Diag_precond_EBE_setup", "ILUp": "ILUp_precond_setup",
                                 "SPIKE": "SPIKE_precond_setup", "NO": "NO_precond_setup"}[kind])

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

    def csr_assembly(self, A):
        """What Build_K_F_SUPG does with CSR storage: one call per element."""
        L = shim()
        A = np.ascontiguousarray(A, dtype=np.float64).reshape(-1, 9)
        for e in range(A.shape[0]):
            L.csr_assembly(*self.ptrs(), e, A[e].ctypes.data)

    def csrmv(self, P):
        Pv = np.array(P, dtype=np.float64, copy=True)
        Q = np.zeros_like(Pv)
        rc = shim().csrmv(*self.ptrs(), Pv.ctypes.data, Q.ctypes.data)
        return rc, Q


# ---------------------------------------------------------------------------
# The multi-dof drivers: libfemgpu_ns.so (steady Navier-Stokes, NDOF = 3) and
# libfemgpu_euler.so (Euler, NDOF = 4), whose structs are restated in
# compat/femgpu_ref_ns.h and compat/femgpu_ref_euler.h
# (SSNavierStokesEquations.h:16-165, EulerEquations.h:16-201).

def _node_type(ndof):
    class Node(ctypes.Structure):
        _fields_ = [("x", c_dbl), ("y", c_dbl), ("Type", c_int * ndof), ("Send", c_int * ndof),
                    ("invP_id", c_int * ndof)]
    return Node


NSNodeType, EulerNodeType = _node_type(3), _node_type(4)

_INT_TAIL = ["KrylovBasisVectorsQuantity", "nnodes", "nNodes", "nel", "nEl", "neq", "neq_bef", "neqaux_bef",
             "neqaux_aft", "nsend_bef", "nsend_aft", "nrecv_bef", "nrecv_aft", "NEQ"]
_INT_END = ["nnzero", "nnzero_bef", "nnzero_aft", "iterations", "k_SPIKE_block_size", "RANK", "NPROC",
            "LinearMaxIter", "NonLinearMaxIter", "bandwidth_bef", "bandwidth_aft"]


class NSParametersType(ctypes.Structure):
    _fields_ = [(n, c_char * 200) for n in ("ProblemTitle", "Solver", "MatrixVectorProductScheme",
                                            "StabilizationForm", "Preconditioner", "Experiments", "reordering")] + \
               [(n, c_dbl) for n in ("SolverTolerance", "NonLinearTolerance", "ReynoldsNumber")] + \
               [(n, c_int) for n in _INT_TAIL + _INT_END] + [("PardisoVariables", ctypes.c_void_p)]


class EulerParametersType(ctypes.Structure):
    _fields_ = [(n, c_char * 200) for n in ("ProblemTitle", "Solver", "TimeIntegration", "MatrixVectorProductScheme",
                                            "StabilizationForm", "ShockCapture", "Preconditioner", "Scaling",
                                            "Experiments", "StopMulticorrection", "reordering", "Dimensionless",
                                            "StopAtSteadyState")] + \
               [(n, c_dbl) for n in ("SolverTolerance", "NonLinearTolerance", "TimeIntegrationTolerance",
                                     "StabilizationTolerance", "Mach", "Alpha", "Alpha_Build", "DeltaT",
                                     "DeltaT_Build", "FinalTime", "CurrentTime")] + [("invY", c_dbl * 4)] + \
               [(n, c_int) for n in _INT_TAIL + ["neqrho"] + _INT_END] + [("PardisoVariables", ctypes.c_void_p)]


class BlockMatrixDataType(ctypes.Structure):
    _fields_ = [("A", ctypes.POINTER(P_dbl)), ("Aaux", P_dbl), ("AA", P_dbl), ("AA_bef", P_dbl), ("AA_aft", P_dbl),
                ("Diag", P_dbl), ("invDiag", P_dbl)] + \
               [(n, ctypes.c_void_p) for n in ("BlockDiag", "BlockDiagAux", "invBlockDiag", "invBlockDiagAux",
                                               "invDe", "invDeaux", "LUe", "LUeaux", "Id", "IdAux",
                                               "Scheme_by_Element", "Scheme_by_Element_bef", "Scheme_by_Element_aft",
                                               "order", "JA", "IA", "JA_bef", "IA_bef", "JA_aft", "IA_aft",
                                               "aux_bef", "aux_aft", "ILUp", "mat", "Ailu", "Perm", "invPerm",
                                               "fullC", "fullCaux", "fullB", "fullBaux", "A_SPIKE", "B_SPIKE",
                                               "C_SPIKE", "S_SPIKE")]


_BUFS = [("SendBuffer_bef", P_dbl * 2), ("SendBuffer_aft", P_dbl * 2), ("RecvBuffer_bef", P_dbl * 2),
         ("RecvBuffer_aft", P_dbl * 2)] + [(n, P_int) for n in ("IdSend_bef", "IdSend_aft", "IdRecv_bef", "IdRecv_aft")]


class NSFemStructsType(ctypes.Structure):
    _fields_ = [("lm", ctypes.POINTER(P_int)), ("lmaux", P_int), ("Node", ctypes.POINTER(NSNodeType)),
                ("Element", ctypes.POINTER(ElementType))] + \
               [(n, P_dbl) for n in ("F", "U", "u", "f", "uB", "delta_old")] + [("AuxBuild", ctypes.c_void_p)] + _BUFS


class EulerFemStructsType(ctypes.Structure):
    _fields_ = [("lm", ctypes.POINTER(P_int)), ("lmaux", P_int), ("eqrho", P_int),
                ("Node", ctypes.POINTER(EulerNodeType)), ("Element", ctypes.POINTER(ElementType))] + \
               [(n, P_dbl) for n in ("F", "U", "u", "du", "f", "uB", "duB", "delta_old")] + \
               [("AuxBuild", ctypes.c_void_p)] + _BUFS


class NSFemFunctionsType(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("v1presc", "v2presc", "ppresc", "f1ext", "f2ext", "assembly", "mv",
                                               "precond", "precondR", "precond_setup")]


class EulerFemFunctionsType(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("gamma", "cv", "rhopresc", "v1presc", "v2presc", "epresc",
                                               "InitialSolution", "ShockCapture", "Ax_Ay_calculations", "BC_theta",
                                               "BC_no_penetrability", "BC_General_theta", "StopCriteria",
                                               "StopTimeIntegration", "assembly", "mv", "precond", "precondR",
                                               "precond_setup", "scaling", "unscaling")]


_KINDS = {
    "ns": dict(ndof=3, P=NSParametersType, S=NSFemStructsType, F=NSFemFunctionsType, Node=NSNodeType,
               lib="COMPAT_NS", mv="ebemvNDOF3", bd="BlockDiagDOF3_precond",
               bd_setup="BlockDiagDOF3_precond_EBE_setup", layout="fgc_ns_layout"),
    "euler": dict(ndof=4, P=EulerParametersType, S=EulerFemStructsType, F=EulerFemFunctionsType,
                  Node=EulerNodeType, lib="COMPAT_EULER", mv="ebemvNDOF4", bd="BlockDiag_precond",
                  bd_setup="BlockDiag_precond_EBE_setup", layout="fgc_euler_layout"),
}


def block_layout_offsets(kind):
    """The 31 numbers fgc_ns_layout / fgc_euler_layout and the reference
    harnesses report (sizes and the offsets the shim reads)."""
    k = _KINDS[kind]
    P, M, S, F, N = k["P"], BlockMatrixDataType, k["S"], k["F"], k["Node"]
    return [ctypes.sizeof(P), P.SolverTolerance.offset, P.KrylovBasisVectorsQuantity.offset, P.nnodes.offset,
            P.nel.offset, P.neq.offset, P.neq_bef.offset, P.NEQ.offset, P.iterations.offset, P.RANK.offset,
            P.NPROC.offset, P.LinearMaxIter.offset, P.PardisoVariables.offset, ctypes.sizeof(M), M.Aaux.offset,
            M.Diag.offset, M.invDiag.offset, M.Id.offset, M.A_SPIKE.offset, ctypes.sizeof(S), S.Node.offset,
            S.Element.offset, S.IdRecv_aft.offset, ctypes.sizeof(F), F.mv.offset, F.precond.offset,
            F.precondR.offset, F.precond_setup.offset, ctypes.sizeof(N), N.invP_id.offset, ctypes.sizeof(ElementType)]


_block_shims = {}


def block_shim(kind):
    """libfemgpu_ns.so or libfemgpu_euler.so (built with the package)."""
    if kind not in _block_shims:
        _build.build()
        k = _KINDS[kind]
        L = ctypes.CDLL(getattr(_build, k["lib"]))
        L.pgmres.argtypes = [ctypes.c_void_p] * 6
        for name in (k["mv"], k["bd"], "Diag_precond", "NO_precond"):
            getattr(L, name).argtypes = [ctypes.c_void_p] * 5
        for name in (k["bd_setup"], "Diag_precond_EBE_setup", "NO_precond_setup"):
            getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_int, ctypes.c_void_p]
        getattr(L, k["layout"]).argtypes = [np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")]
        getattr(L, k["layout"]).restype = None
        _block_shims[kind] = L
    return _block_shims[kind]


class BlockDriverState:
    """The structs the NS or Euler Preprocess.c fills for one rank (EBE
    storage, block-diagonal / Diag / no preconditioning, GMRES)."""

    def __init__(self, kind, mesh, kmax=30, lmax=1000, tol=1e-10, precond="BlockDiag"):
        k = _KINDS[kind]
        self.kind, self.k = kind, k
        L = block_shim(kind)
        ndof, S2 = k["ndof"], (3 * k["ndof"]) ** 2
        n, nel, nn = mesh.neq, mesh.nel, mesh.nnodes
        self.P = k["P"]()
        for key, v in (("Solver", b"GMRES"), ("Preconditioner", precond.encode()), ("reordering", b"NOT"),
                       ("MatrixVectorProductScheme", b"EBE")):
            setattr(self.P, key, v)
        self.P.SolverTolerance, self.P.KrylovBasisVectorsQuantity, self.P.LinearMaxIter = tol, kmax, lmax
        self.P.nnodes = self.P.nNodes = nn
        self.P.nel = self.P.nEl = nel
        self.P.neq = self.P.NEQ = n
        self.P.NPROC = 1
        self.nodes = (k["Node"] * nn)()
        t = mesh.type.reshape(nn, ndof)
        ip = mesh.invp.reshape(nn, ndof)
        for i in range(nn):
            self.nodes[i].x, self.nodes[i].y = float(mesh.x[i]), float(mesh.y[i])
            for d in range(ndof):
                self.nodes[i].Type[d] = int(t[i, d])
                self.nodes[i].Send[d] = 1
                self.nodes[i].invP_id[d] = int(ip[i, d]) if t[i, d] else -1
        self.elems = (ElementType * nel)()
        for e in range(nel):
            for v in range(3):
                self.elems[e].Vertex[v] = int(mesh.ien[e, v])
        self.Aaux = np.zeros(nel * S2)
        self.rows = (P_dbl * nel)(*[ctypes.cast(self.Aaux.ctypes.data + 8 * S2 * e, P_dbl) for e in range(nel)])
        self.Diag = np.zeros(n + 1)
        self.invDiag = np.zeros(n + 1)
        self.M = BlockMatrixDataType()
        self.M.A = ctypes.cast(self.rows, ctypes.POINTER(P_dbl))
        self.M.Aaux = self.Aaux.ctypes.data_as(P_dbl)
        self.M.Diag = self.Diag.ctypes.data_as(P_dbl)
        self.M.invDiag = self.invDiag.ctypes.data_as(P_dbl)
        self.S = k["S"]()
        self.S.Node = ctypes.cast(self.nodes, ctypes.POINTER(k["Node"]))
        self.S.Element = ctypes.cast(self.elems, ctypes.POINTER(ElementType))
        self.Fn = k["F"]()
        self.Fn.mv = _addr(L, k["mv"])
        pc = {"BlockDiag": (k["bd"], k["bd_setup"]), "Diag": ("Diag_precond", "Diag_precond_EBE_setup"),
              "NOT": ("NO_precond", "NO_precond_setup")}[precond]
        self.Fn.precond = _addr(L, pc[0])
        self.Fn.precondR = _addr(L, "NO_precond")
        self.setup = getattr(L, pc[1])

    def ptrs(self):
        return (ctypes.addressof(self.P), ctypes.addressof(self.M), ctypes.addressof(self.S))

    def precond_setup(self, F, tag=1):
        F = np.array(F, dtype=np.float64, copy=True)
        rc = self.setup(*self.ptrs(), tag, F.ctypes.data)
        return rc, F

    def pgmres(self, B):
        B = np.ascontiguousarray(B, dtype=np.float64)
        X = np.zeros_like(B)
        rc = block_shim(self.kind).pgmres(*self.ptrs(), ctypes.addressof(self.Fn), B.ctypes.data, X.ctypes.data)
        return rc, X

    def ebemv(self, P):
        Pv = np.array(P, dtype=np.float64, copy=True)
        Q = np.zeros_like(Pv)
        rc = getattr(block_shim(self.kind), self.k["mv"])(*self.ptrs(), Pv.ctypes.data, Q.ctypes.data)
        return rc, Q
