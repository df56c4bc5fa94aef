"""Parity at the sizes and settings of the benchmark configurations.

* Steady transport 129 x 129 nodes, velocity (cos 30, sin 30), k = 1e-6,
  SUPG + CAU, Diag, GMRES(30), tol 1e-10: the plain FP64 GPU solve against
  the oracle's restatement of pgmres.c:5-200 (rel-L2 <= 1e-9, iterations
  within +-2), the mixed-precision solve against the oracle's matvec (true
  residual <= 1e-10) and the whole CAU Process loop
  (01_SS_Transport_Equation/2D/01_CommonFiles/Process.c:6-93).
* Euler OBLIQUO 65 x 65 nodes, 3 steps of Predictor_Old with 2
  corrections (00_CommonFiles/Time_Integration/Predictor_Old.c:53-123),
  GMRES(25), BlockDiag: u and a against the oracle's loop to 1e-8.
* Navier-Stokes lid-driven cavity 65 x 65 nodes, interior jittered by
  0.2 h (seed 3), Re = 1000, one Picard step
  (04_SS_NavierStokes_Equations/2D/01_CommonFiles/Process.c:33-52),
  GMRES(50), BlockDiagDOF3: the solution against the oracle's.
"""
import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def fg():
    from parallel_fem_codes_gb300 import femgpu
    femgpu.lib()
    return femgpu


@pytest.fixture(scope="module")
def c1():
    p = G.transport_problem(129, angle_deg=30.0, k=1e-6)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    X0, it0, _, _, Fp0 = O.ebe_diag_solve(lm, A, m.neq, F, perm, inv, kmax=30, lmax=1000, tol=1e-10)
    return p, A, F, lm, perm, inv, X0, it0


def test_c1_plain_fp64_gmres(fg, c1):
    p, A, F, lm, perm, inv, X0, it0 = c1
    s = fg.System(p.mesh)
    s.set_blocks(A)
    Fp = s.precond_setup(fg.FG_PRECOND_DIAG, 0, F)
    r = s.solve(Fp, kmax=30, lmax=1000, tol=1e-10, F_true=F)
    assert r.stats["converged"] == 1 and r.stats["status"] == 0
    assert abs(r.stats["iterations"] - it0) <= 2
    assert rel(r.x[:-1], X0[:-1]) <= 1e-9


def test_c1_mixed_reaches_true_residual(fg, c1):
    p, A, F, lm, perm, inv, X0, it0 = c1
    s = fg.System(p.mesh)
    s.set_blocks(A)
    Fp = s.precond_setup(fg.FG_PRECOND_DIAG, 0, F)
    r = s.solve(Fp, tol=1e-10, F_true=F, precision=fg.FG_PREC_MIXED)
    assert r.stats["converged"] == 1
    res = np.linalg.norm(F[:-1] - O.ebemv3_perm(lm, A, perm, inv, r.x)[:-1]) / np.linalg.norm(F[:-1])
    assert res <= 1e-10
    # error against the FP64 oracle solution: the residual bound times the
    # conditioning of this convection-dominated system
    assert rel(r.x[:-1], X0[:-1]) <= 1e-7


def test_c1_device_assembly_and_process(fg, c1):
    p, A, F, *_ = c1
    s = fg.transport_system(p)
    Fd = s.transport_assemble(p)
    assert np.array_equal(s.get_blocks(), A) and np.array_equal(Fd[:-1], F[:-1])
    U0, nl0, it0 = O.transport_process(p, 1e-10, 1e-3, 30, 1000)
    U, st = s.transport_process(p, 30, 1000, 1e-10, 1e-3)
    assert st["nonlinear_iterations"] == nl0
    # three nonlinear iterations of ~560 GMRES steps each on a near-stagnating
    # convection-dominated system: totals agree to 2%
    assert abs(st["gmres_iterations"] - it0) <= max(2 * nl0, it0 // 50)
    assert rel(U, U0) <= 1e-9


@pytest.mark.parametrize("precision", [64, 32])
def test_euler_obliquo65_predictor(fg, precision):
    p = G.obliquo_problem(65)
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt, 1e-6, 0)
    uo, ao, sto = O.euler_predictor(p, to_o, tol=1e-10, kmax=25)
    s = fg.euler_system(p)
    ug, ag, st = s.euler_predictor(p, fg.time_opts(0, 2, 1e-3, 0, 3 * p.dt, 1e-6), kmax=25, tol=1e-10,
                                   precision=fg.FG_PREC_FP64 if precision == 64 else fg.FG_PREC_MIXED)
    assert st["steps"] == sto["steps"] == 3 and st["corrections"] == sto["corrections"] == 6
    # FP64 stops on the reference's preconditioned estimate (pgmres.c:155-159),
    # the mixed path on the true residual
    assert st["true_rel_residual"] <= (1e-10 if precision == 32 else 1e-8)
    assert rel(ug, uo) <= 1e-8
    assert rel(ag, ao) <= 1e-8
    if precision == 64:
        assert abs(st["gmres_iterations"] - sto["gmres_iterations"]) <= 2 * 6


def test_ns_cavity65_one_picard_step(fg):
    p = G.cavity_problem(65, reynolds=1000.0, jitter=0.2)
    uo, nl_o, its_o, last_o = O.ns_process(p, 1e-10, 1e-6, 50, 1000, 1)
    s = fg.ns_system(p)
    ug, st = s.ns_process(p, kmax=50, lmax=1000, tol=1e-10, nonlinear_tol=1e-6, max_nonlinear=1)
    assert st["nonlinear_iterations"] == nl_o == 1
    # tens of thousands of GMRES(50) steps: counts agree to 1%
    assert abs(st["gmres_iterations"] - its_o) <= max(2, its_o // 100)
    assert rel(ug, uo) <= 1e-9
