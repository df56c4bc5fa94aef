"""The reference's own drivers, linked unchanged against the drop-in shims
(oracle/Makefile `dropin`), run on the GPU and agree with the same drivers
linked with the reference's CPU solve path (oracle/Makefile `ref`):

* steady transport Process.c (01_SS_Transport_Equation/2D/01_CommonFiles/
  Process.c:6-93: CAU fixed point, Diag_precond_EBE_setup + pgmres per
  iteration), 33 x 33 nodes;
* Navier-Stokes Process.c (04_SS_NavierStokes_Equations/2D/01_CommonFiles/
  Process.c:6-62: Picard, BlockDiagDOF3 + pgmres), cavity 17 x 17, Re 100;
* Predictor_Old.c (00_CommonFiles/Time_Integration/Predictor_Old.c:6-134:
  Euler OBLIQUO 17 x 17, 4 steps, 2 corrections, BlockDiag + pgmres);
* Predictor_New.c with Build_M_F_DD_Transiente.c ("Predictor2", DD,
  YZBeta: the bubble unknowns, calculate_DaB), 3 steps;
* the transient transport driver (02_Transport_Equation: Predictor_Old.c
  with Build_M_K_R_SUPG / _DD, Predictor_New.c with Build_M_F_DD) against
  libfemgpu_tt.so, 4 steps.

Solutions within rel-L2 1e-9, GMRES iterations (Parameters->iterations)
within +-2 per linear solve.  Skipped where the drop-in builds are absent
(they compile the reference's driver sources).
"""
import os

import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not (O.dropin_available() and O.ref_available()),
                                 reason="drop-in builds of the reference drivers absent")]


# a shim error returns its status instead of ending the test process
os.environ["FEMGPU_COMPAT_NO_EXIT"] = "1"


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_transport_process_dropin():
    p = G.transport_problem(33, angle_deg=30.0, k=1e-6)
    U0, it0 = O.ref_process(p, 1e-10, 1e-3, 30, 1000)
    U1, it1 = O.ref_process(p, 1e-10, 1e-3, 30, 1000, dropin=True)
    assert rel(U1, U0) <= 1e-9
    assert abs(it1 - it0) <= 2 * 10


def test_ns_process_dropin():
    p = G.cavity_problem(17, reynolds=100.0)
    u0, it0 = O.ref_ns_process(p, 1e-10, 1e-6, 30, 1000, 40)
    u1, it1 = O.ref_ns_process(p, 1e-10, 1e-6, 30, 1000, 40, dropin=True)
    assert rel(u1, u0) <= 1e-9
    assert abs(it1 - it0) <= 2 * 40


def test_euler_predictor_old_dropin():
    p = G.obliquo_problem(17)
    to = O.TimeOpts(0, 2, 1e-3, 0, 4 * p.dt, 1e-6, 0)
    u0, it0, t0 = O.ref_euler_predictor(p, to, tol=1e-10, kmax=25)
    u1, it1, t1 = O.ref_euler_predictor(p, to, tol=1e-10, kmax=25, dropin=True)
    assert t1 == t0
    assert rel(u1, u0) <= 1e-9
    assert abs(it1 - it0) <= 2 * 8


def test_euler_predictor2_dropin():
    """Predictor_New.c with Build_M_F_DD_Transiente.c ("Predictor2", DD,
    YZBeta) linked unchanged against the shims."""
    p = G.obliquo_problem(17)
    p.invY = np.array([1.0, 0.5, 2.0, 0.25])
    to = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt + 1e-12, 1e-6, 0, 3)
    u0, it0, _ = O.ref_euler_predictor(p, to, tol=1e-10, kmax=25)
    u1, it1, _ = O.ref_euler_predictor(p, to, tol=1e-10, kmax=25, dropin=True)
    assert rel(u1, u0) <= 1e-9
    assert abs(it1 - it0) <= 2 * 6


@pytest.mark.skipif(not O.dropin_tt_available(), reason="transient-transport drop-in build absent")
@pytest.mark.parametrize("form,cau,scheme", [(0, 1, 0), (1, 2, 0), (1, 2, 3)],
                         ids=["predictor1-supg", "predictor1-dd", "predictor2-dd"])
def test_transient_transport_dropin(form, cau, scheme):
    """The transient driver's Predictor_Old / Predictor_New with its builds,
    linked unchanged against libfemgpu_tt.so, against the same files linked
    with the reference's CPU solve path."""
    p = G.transport_problem(17, angle_deg=30.0, k=1e-3, f=0.0, cau=cau)
    p.form = form
    to = O.TimeOpts(0, 2, 1e-3, 0, 4 * 0.02 + 1e-12, 1e-6, 0, 0)
    run = O.ref_tt_predictor2 if scheme == 3 else O.ref_tt_predictor1
    u0, it0 = run(p, 0.5, 0.02, to)
    u1, it1 = run(p, 0.5, 0.02, to, dropin=True)
    assert rel(u1, u0) <= 1e-9
    assert abs(it1 - it0) <= 2 * 8
