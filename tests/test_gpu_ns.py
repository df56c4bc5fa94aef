"""Steady Navier-Stokes on the GPU against the oracle (pinned bit-exactly to
the reference's NS driver by tests/test_oracle_ns.py) and against the golden
fixtures generated from the reference itself.

The element build (9x9 Picard tangent and residual, FP64, no FMA
contraction) and the BlockDiagDOF3 set-up are bit-exact.  The Picard loop
solves every linear system to tol 1e-10 with CGS2 GMRES instead of MGS, so
the solution agrees to a relative 1e-7 with the same number of nonlinear
iterations (within one); mixed precision reaches the same nonlinear
tolerance and agrees to 1e-6."""
import glob
import os

import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ns_*.npz")))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def fg():
    from parallel_fem_codes_gb300 import femgpu
    femgpu.lib()
    return femgpu


def _affine(seed=5, n=13, re=50.0):
    mesh = G.multi_dof_mesh(n, 3, seed=2, jitter=0.2)
    coef = np.random.Generator(np.random.PCG64(seed)).standard_normal((5, 3))
    return G.ns_problem(mesh, re, coef)


@pytest.mark.parametrize("case", ["cavity17", "cavity33_jitter", "affine13"])
def test_ns_assembly_bit_exact(fg, case):
    if case == "cavity17":
        p = G.cavity_problem(17, reynolds=1000.0)
    elif case == "cavity33_jitter":
        p = G.cavity_problem(33, reynolds=400.0, jitter=0.2)
    else:
        p = _affine()
    u = np.random.default_rng(7).standard_normal(p.mesh.neq)
    A, F = O.build_ns(p, u)
    s = fg.ns_system(p)
    Fg = s.ns_assemble(p, u)
    assert np.array_equal(Fg, F)
    assert np.array_equal(s.get_blocks(), A)
    # at u = 0 as well (the first Picard build)
    A0, F0 = O.build_ns(p)
    assert np.array_equal(s.ns_assemble(p), F0)
    assert np.array_equal(s.get_blocks(), A0)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_ns_golden(fg, path):
    g = dict(np.load(path))
    m = G.Mesh(g["x"], g["y"], g["ien"], 3, g["type"], g["invp"], int(g["neq"]))
    p = G.ns_problem(m, float(g["reynolds"]), g["coef"], bool(g["lid"]))
    s = fg.ns_system(p)
    F = s.ns_assemble(p, g["u"])
    assert np.array_equal(F, g["F"])
    assert np.array_equal(s.get_blocks(), g["A"])
    Fp = s.precond_setup(fg.FG_PRECOND_BLOCKDIAG, 0, F)
    assert np.array_equal(Fp, g["Fp"])
    assert rel(s.matvec(g["P"])[:-1], g["Q"][:-1]) < 1e-14


def test_ns_blockdiag_bit_exact(fg):
    p = G.cavity_problem(33, reynolds=1000.0, jitter=0.2)
    u = np.random.default_rng(3).standard_normal(p.mesh.neq)
    A, F = O.build_ns(p, u)
    bd, ibd, Id, Fo = O.blockdiag_setup(p.mesh, A, F)
    s = fg.ns_system(p)
    Fg = s.ns_assemble(p, u)
    Fp = s.precond_setup(fg.FG_PRECOND_BLOCKDIAG, 0, Fg)
    assert np.array_equal(Fp, Fo)


def test_ns_process_fp64(fg):
    p = G.cavity_problem(17, reynolds=100.0)
    uo, nl_o, its_o, last_o = O.ns_process(p, 1e-10, 1e-6, 30, 1000, 40)
    s = fg.ns_system(p)
    ug, st = s.ns_process(p, kmax=30, tol=1e-10, nonlinear_tol=1e-6, max_nonlinear=40)
    assert abs(st["nonlinear_iterations"] - nl_o) <= 1
    assert st["nonlinear_residual"] <= 1e-6
    assert rel(ug, uo) < 1e-7


@pytest.mark.parametrize("precond", ["ilu0", "spike"])
def test_ns_process_csr_rcm(fg, precond):
    """The Picard loop on the CSR operator in the RCM numbering with ILU(0)
    or SPIKE reaches the oracle's (BlockDiagDOF3) solution."""
    p = G.cavity_problem(17, reynolds=100.0)
    uo, nl_o, its_o, last_o = O.ns_process(p, 1e-10, 1e-6, 30, 1000, 40)
    s = fg.ns_system(p, reorder=True)
    s.set_operator(fg.FG_OP_CSR)
    kind = fg.FG_PRECOND_ILU0 if precond == "ilu0" else fg.FG_PRECOND_SPIKE
    if precond == "spike":
        s.set_spike(12, 4)
    ug, st = s.ns_process(p, kmax=30, tol=1e-10, nonlinear_tol=1e-6, max_nonlinear=40, precond=kind)
    assert abs(st["nonlinear_iterations"] - nl_o) <= 1
    assert st["nonlinear_residual"] <= 1e-6
    assert rel(ug, uo) < 1e-7


def test_ns_process_mixed(fg):
    p = G.cavity_problem(17, reynolds=100.0, jitter=0.2)
    uo, nl_o, its_o, last_o = O.ns_process(p, 1e-10, 1e-6, 30, 1000, 40)
    s = fg.ns_system(p)
    ug, st = s.ns_process(p, kmax=30, tol=1e-10, nonlinear_tol=1e-6, max_nonlinear=40,
                          precision=fg.FG_PREC_MIXED)
    assert st["nonlinear_residual"] <= 1e-6
    assert rel(ug, uo) < 1e-6


def test_ns_process_from_state(fg):
    """Restarting from the converged state takes one iteration and moves
    nothing beyond the tolerance."""
    p = G.cavity_problem(17, reynolds=100.0)
    s = fg.ns_system(p)
    u1, st1 = s.ns_process(p, nonlinear_tol=1e-8, max_nonlinear=60)
    u2, st2 = s.ns_process(p, u0=u1, nonlinear_tol=1e-8, max_nonlinear=60)
    assert st2["nonlinear_iterations"] == 1
    assert rel(u2, u1) <= 1e-8


def test_ns_rejects_scalar_system(fg):
    p = G.transport_problem(9)
    s = fg.System(p.mesh)
    with pytest.raises(fg.FemGpuError):
        s.ns_set_geometry(G.ns_problem(G.multi_dof_mesh(9, 3), 10.0))


@pytest.mark.parametrize("case", ["cavity33_jitter", "affine13"])
def test_ns_vms_dcdd_assembly_bit_exact(fg, case):
    """Build_K_F_VMS_DCDD on the device against the oracle (pinned to the
    reference's build): blocks and residual bit-identical."""
    p = G.cavity_problem(33, reynolds=400.0, jitter=0.2) if case == "cavity33_jitter" else _affine()
    u = np.random.default_rng(9).standard_normal(p.mesh.neq)
    A, F = O.build_ns(p, u, form=1)
    s = fg.ns_system(p)
    assert np.array_equal(s.ns_assemble(p, u, form=fg.FG_NS_VMS_DCDD), F)
    assert np.array_equal(s.get_blocks(), A)


def test_ns_vms_dcdd_process(fg):
    p = G.cavity_problem(17, reynolds=100.0)
    uo, nl_o, its_o, last_o = O.ns_process(p, 1e-10, 1e-6, 30, 1000, 40, form=1)
    s = fg.ns_system(p)
    ug, st = s.ns_process(p, kmax=30, tol=1e-10, nonlinear_tol=1e-6, max_nonlinear=40, form=fg.FG_NS_VMS_DCDD)
    assert abs(st["nonlinear_iterations"] - nl_o) <= 1
    assert st["nonlinear_residual"] <= 1e-6
    assert rel(ug, uo) < 1e-7
