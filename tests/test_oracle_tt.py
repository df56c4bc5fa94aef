"""The transient transport restatement (oracle/tt.c: Build_M_K_R_SUPG.c,
Build_M_K_R_DD.c and the Predictor_Old loop with Diag).

Pinned to the reference itself: the transient driver's TranspEquation.h
includes an MPI header by absolute path (line 8), so oracle/Makefile
(`ref_tt`) compiles its build functions from a private copy with that line
pointed at the MPI stand-in; tests/golden/tt_ref.npz holds that build's
blocks and residuals (SUPG with CAU / YZBeta and each h_shock option, DD
with CAUDD / YZBeta) at random states, and the restatement matches them
bit for bit.  The checks through the steady build (pinned against the
reference's steady driver) and the time-loop properties below stay."""
import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G


def test_stiffness_part_equals_steady_block():
    p = G.transport_problem(17, angle_deg=35.0, k=1e-3, gamma=0.2, f=0.5)
    u = np.random.default_rng(0).random(p.mesh.neq)
    K, _ = O.build_k_f_supg(p, u)
    A1, _ = O.build_tt(p, 0.5, 2.0, u=u)        # me + 1 * ke
    A2, _ = O.build_tt(p, 0.5, 4.0, u=u)        # me + 2 * ke
    scale = np.abs(K).max()
    assert np.abs((A2 - A1) - K).max() <= 1e-13 * scale
    # the mass part (A1 - K) is the consistent P1 mass plus the SUPG term
    me = 2 * A1 - A2
    assert np.all(np.abs(me).max(axis=1) > 0)


def test_load_part_equals_steady_rhs():
    """u = 0, du = 0, zero Dirichlet data: R is the SUPG load, which the
    steady build assembles the same way (no lifting when the data are 0)."""
    p = G.transport_problem(17, angle_deg=10.0, k=1e-4, f=1.0, upmode=1, upval=0.0)
    _, F = O.build_k_f_supg(p)
    _, R = O.build_tt(p, 0.5, 0.1)
    assert np.array_equal(R[:-1], F[:-1]) and R[-1] == 0.0


def test_residual_of_du_is_mass_times_du():
    """Linear in du: R(u, du) - R(u, 0) = -me du, with the element order of
    the reference's accumulation (checked to rounding)."""
    p = G.transport_problem(9, angle_deg=60.0, k=1e-2, cau=False)
    rng = np.random.default_rng(3)
    u = rng.random(p.mesh.neq)
    du = rng.random(p.mesh.neq)
    _, R0 = O.build_tt(p, 0.5, 0.1, u=u)
    _, R1 = O.build_tt(p, 0.5, 0.1, u=u, du=du)
    A1, _ = O.build_tt(p, 0.5, 2.0, u=u)
    A2, _ = O.build_tt(p, 0.5, 4.0, u=u)
    me = 2 * A1 - A2
    lm = O.fill_lm(p.mesh)
    Mdu = O.ebemv(lm, me, p.mesh.neq, np.append(du, 0.0))
    assert np.abs((R0 - R1)[:-1] - Mdu[:-1]).max() <= 1e-12 * np.abs(Mdu).max()


def test_constant_state_is_kept():
    """u = c everywhere with f = gamma c is a steady solution (TESTE)."""
    c, gamma = 2.5, 0.3
    p = G.transport_problem(17, angle_deg=30.0, k=1e-3, gamma=gamma, f=gamma * c, upmode=1, upval=c)
    u0 = np.full(p.mesh.neq, c)
    u, a, st = O.tt_predictor(p, 0.5, 0.01, O.TimeOpts(0, 2, 1e-3, 0, 0.05, 1e-6, 0), u0=u0)
    assert st["steps"] == 5
    assert np.abs(u - c).max() <= 1e-10 and np.abs(a).max() <= 1e-8


def test_reaches_the_steady_solution():
    p = G.transport_problem(17, angle_deg=30.0, k=1e-2, cau=False)
    Us, nl, its = O.transport_process(p, 1e-12, 1e-3, 30, 1000)
    u, a, st = O.tt_predictor(p, 0.5, 0.05, O.TimeOpts(1, 5, 1e-6, 1, 1e3, 1e-9, 0), tol=1e-12)
    assert np.linalg.norm(u - Us[: p.mesh.neq]) / np.linalg.norm(Us[: p.mesh.neq]) < 1e-6


def test_tt_dd_pinned_through_steady_dd(oracle_lib):
    """The transient DD build (Build_M_K_R_DD) against the steady DD build
    (pinned bit-exactly to the reference's Build_K_F_DD): at u = du = 0 with
    zero boundary data the load is bit-identical; the stiffness part
    (Ae(dt1) - Ae(dt2)) / (alpha (dt1 - dt2)) equals the steady block to
    rounding; the mass part is Mhh (1 + delta_ij) - KhB MBh / KBB."""
    p = G.transport_problem(13, angle_deg=110.0, k=1e-3, gamma=0.3, f=0.7, upmode=1, upval=0.0, cau=0)
    p.form = 1
    A_ss, F_ss = O.build_k_f_supg(p)
    A1, R1 = O.build_tt(p, 0.5, 0.1)
    A2, R2 = O.build_tt(p, 0.5, 0.05)
    assert np.array_equal(R1[:-1], F_ss[:-1])
    ke = (A1 - A2) / (0.5 * (0.1 - 0.05))
    assert np.allclose(ke, A_ss, rtol=1e-9, atol=1e-12 * np.abs(A_ss).max())


def test_tt_dd_caudd_state_and_loop(oracle_lib):
    """CAUDD in the transient DD build: the relaxed coefficient depends on the
    previous build (state), and the Predictor_Old loop converges to the
    steady DD solution of the same problem."""
    p = G.transport_problem(13, angle_deg=30.0, k=1e-2, cau=2)
    p.form = 1
    u = np.random.default_rng(3).random(p.mesh.neq)
    A1, _ = O.build_tt(p, 0.5, 0.05, u=u)
    A2, _ = O.build_tt(p, 0.5, 0.05, u=u)
    assert np.array_equal(A1, A2)                    # fresh state each single build
    uo, ao, st = O.tt_predictor(p, 0.5, 0.5, O.TimeOpts(1, 5, 1e-8, 1, 1e4, 1e-9, 0), tol=1e-12)
    Us, nl, its = O.transport_process(p, 1e-12, 1e-8, 30, 1000)
    assert np.linalg.norm(uo - Us) <= 1e-5 * np.linalg.norm(Us)


@pytest.mark.parametrize("hs", [0, 1, 2])
def test_tt_yzbeta_pinned_through_steady_yzbeta(oracle_lib, hs):
    """YZBeta_ShockCapture of the transient driver (no state, Ru with du/dt)
    against the steady driver's (reference-pinned; relaxed with w = 1/2 on a
    fresh state): at du = 0 the transient shock coefficient is twice the
    steady first-build one, so the shock part of the stiffness doubles, for
    each h_shock option.  Two transient builds at the same state agree
    bit-for-bit (no state)."""
    u = np.random.default_rng(7).random(G.transport_problem(13).mesh.neq)

    def stiff(cau):
        p = G.transport_problem(13, angle_deg=40.0, k=1e-3, gamma=0.2, f=0.5, cau=cau)
        p.h_shock = hs
        A1, _ = O.build_tt(p, 0.5, 0.1, u=u)
        A2, _ = O.build_tt(p, 0.5, 0.05, u=u)
        A1b, _ = O.build_tt(p, 0.5, 0.1, u=u)
        assert np.array_equal(A1, A1b)
        Ass, _ = O.build_k_f_supg(p, u=u)
        return (A1 - A2) / (0.5 * (0.1 - 0.05)), Ass

    ke3, ks3 = stiff(3)
    ke0, ks0 = stiff(0)
    shock_tt, shock_ss = ke3 - ke0, ks3 - ks0
    assert np.abs(shock_ss).max() > 0
    assert np.allclose(shock_tt, 2 * shock_ss, rtol=1e-7, atol=1e-9 * np.abs(ke0).max())


TT_CASES = [(0, 1, 0), (0, 3, 1), (0, 1, 2), (1, 2, 0), (1, 3, 2)]   # (form, shock, h_shock)


def _tt_problem(form, cau, hs):
    p = G.transport_problem(17, angle_deg=35.0, k=1e-3, gamma=0.2, f=0.5, cau=cau)
    p.form, p.h_shock = form, hs
    return p


@pytest.mark.parametrize("form,cau,hs", TT_CASES)
def test_transient_build_matches_reference_golden(form, cau, hs):
    """Blocks and residual bit-identical with the reference's own transient
    build (tests/golden/tt_ref.npz, written by tests/golden/make_golden.py)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "tt_ref.npz"))
    key = f"tt_{form}_{cau}_{hs}"
    A, R = O.build_tt(_tt_problem(form, cau, hs), 0.5, 0.01, g[key + "_u"], g[key + "_du"])
    assert np.array_equal(A, g[key + "_A"])
    assert np.array_equal(R[:-1], g[key + "_R"][:-1])


@pytest.mark.skipif(O.ref_tt() is None, reason="reference transient build absent")
@pytest.mark.parametrize("form,cau,hs", TT_CASES)
def test_transient_build_matches_reference(form, cau, hs):
    p = _tt_problem(form, cau, hs)
    rng = np.random.default_rng(7)
    u, du = rng.random(p.mesh.neq), rng.standard_normal(p.mesh.neq)
    A0, R0 = O.build_tt(p, 0.3, 0.05, u, du)
    A1, R1 = O.ref_tt_build(p, 0.3, 0.05, u, du)
    assert np.array_equal(A0, A1) and np.array_equal(R0[:-1], R1[:-1])


# ---- TimeIntegration "Predictor2" with the DD form: Build_M_F_DD.c,
# calculate_DaB.c and Predictor_New.c (the bubble of each element kept as
# an unknown and condensed out of the element system) ----

P2_CASES = [(2, 0), (3, 2)]    # (shock CAUDD / YZBeta, h_shock)


def _p2_problem(cau, hs, n=17):
    p = G.transport_problem(n, angle_deg=35.0, k=1e-3, gamma=0.2, f=0.5, cau=cau)
    p.form, p.h_shock = 1, hs
    return p


@pytest.fixture(scope="module")
def p2gold():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "tt_predictor2_ref.npz"))


@pytest.mark.parametrize("cau,hs", P2_CASES)
def test_predictor2_build_matches_reference_golden(p2gold, cau, hs):
    """Me, F, the condensation data (invN2, R2, M2) and calculate_DaB's
    bubble increments bit-identical with the reference's own functions."""
    g, key = p2gold, f"p2_{cau}_{hs}"
    p = _p2_problem(cau, hs)
    A, F, cond = O.build_tt_mfdd(p, 0.5, 0.01, g[key + "_u"], g[key + "_du"], g[key + "_uB"], g[key + "_duB"])
    assert np.array_equal(A, g[key + "_A"])
    assert np.array_equal(F, g[key + "_F"])
    assert np.array_equal(cond, g[key + "_cond"])
    DaB = O.tt_dab(O.fill_lm(p.mesh), cond, g[key + "_Da"])
    assert np.array_equal(DaB, g[key + "_DaB"])


@pytest.mark.parametrize("cau,hs", P2_CASES)
def test_predictor2_loop_matches_reference_golden(p2gold, cau, hs):
    """The whole Predictor_New loop (4 steps x 2 corrections, Diag, GMRES):
    the final state and the GMRES iteration count equal the reference's."""
    g, key = p2gold, f"p2_{cau}_{hs}"
    to = O.TimeOpts(0, 2, 1e-3, 0, 0.04 + 1e-12, 1e-6, 0, 0)
    u, a, uB, aB, st = O.tt_predictor2(_p2_problem(cau, hs), 0.5, 0.01, to, tol=1e-10, kmax=30, lmax=1000)
    assert st["steps"] == 4 and st["corrections"] == 8
    assert st["gmres_iterations"] == int(g[key + "_its"][0])
    assert np.array_equal(u, g[key + "_U"])


@pytest.mark.skipif(O.ref_tt() is None, reason="reference transient build absent")
def test_predictor2_matches_reference_live():
    p = _p2_problem(2, 1, n=13)
    m = p.mesh
    rng = np.random.default_rng(11)
    u, du = rng.random(m.neq), rng.standard_normal(m.neq)
    uB, duB = rng.random(m.nel), rng.standard_normal(m.nel)
    Da = np.append(rng.standard_normal(m.neq), 1.0)
    A0, F0, c0, D0 = O.ref_tt_mfdd_build(p, 0.3, 0.05, u, du, uB, duB, Da)
    A1, F1, c1 = O.build_tt_mfdd(p, 0.3, 0.05, u, du, uB, duB)
    assert np.array_equal(A0, A1) and np.array_equal(F0, F1) and np.array_equal(c0, c1)
    assert np.array_equal(D0, O.tt_dab(O.fill_lm(m), c1, Da))
    to = O.TimeOpts(1, 3, 1e-4, 0, 0.15 + 1e-12, 1e-6, 0, 0)
    U0, its0 = O.ref_tt_predictor2(p, 0.5, 0.05, to, tol=1e-10)
    U1, a1, uB1, aB1, st = O.tt_predictor2(p, 0.5, 0.05, to, tol=1e-10)
    assert st["gmres_iterations"] == its0 and np.array_equal(U0, U1)


def test_predictor2_bubble_condensation():
    """Static condensation: the condensed element system is exact.  For
    each element, solving the 4x4 system [M1 N1; M2 N2] (nodal rows and the
    bubble row) for (Da_e, DaB) with the element's own residuals gives
    DaB = invN2 (R2 - M2 . Da_e), and Me Da_e = R1 - N1 invN2 R2 on the
    nodal rows -- checked by assembling the 4x4 blocks from the
    condensation data and comparing with calculate_DaB's increments."""
    p = _p2_problem(2, 0, n=9)
    m = p.mesh
    rng = np.random.default_rng(5)
    A, F, cond = O.build_tt_mfdd(p, 0.5, 0.02, rng.random(m.neq), rng.standard_normal(m.neq),
                                 rng.random(m.nel), rng.standard_normal(m.nel))
    Da = np.append(rng.standard_normal(m.neq), 0.0)
    DaB = O.tt_dab(O.fill_lm(m), cond, Da)
    lm = O.fill_lm(m)
    invN2, R2, M2 = cond[:, 0], cond[:, 1], cond[:, 2:5]
    # bubble row of the 4x4 system: M2 . Da_e + N2 DaB = R2
    resid = np.einsum("ej,ej->e", M2, Da[lm]) + DaB / invN2 - R2
    assert np.abs(resid).max() <= 1e-12 * max(np.abs(R2).max(), 1.0)


def test_predictor2_reaches_the_steady_dd_solution():
    """With a large step the loop's state approaches the steady DD solution
    of the same problem (the bubble equation is the steady DD's in the
    limit du/dt -> 0)."""
    p = _p2_problem(2, 0, n=13)
    p.k = 1e-2
    u, a, uB, aB, st = O.tt_predictor2(p, 0.5, 0.5, O.TimeOpts(1, 5, 1e-8, 1, 1e4, 1e-9, 0, 0), tol=1e-12)
    Us, nl, its = O.transport_process(p, 1e-12, 1e-8, 30, 1000)
    assert np.linalg.norm(u - Us[: p.mesh.neq]) <= 1e-4 * np.linalg.norm(Us[: p.mesh.neq])


@pytest.mark.parametrize("form,cau", [(0, 1), (1, 2)], ids=["supg-cau", "dd-caudd"])
def test_predictor1_loop_matches_reference_golden(form, cau):
    """The Predictor_Old loop of the transient driver (Diag, GMRES) with the
    SUPG and DD builds: final state and GMRES iterations equal the
    reference's own loop (tests/golden/tt_predictor1_ref.npz)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "tt_predictor1_ref.npz"))
    p = G.transport_problem(17, angle_deg=30.0, k=1e-3, f=0.0, cau=cau)
    p.form = form
    to = O.TimeOpts(0, 2, 1e-3, 0, 4 * 0.02 + 1e-12, 1e-6, 0, 0)
    u, a, st = O.tt_predictor(p, 0.5, 0.02, to)
    assert st["gmres_iterations"] == int(g[f"p1_{form}_its"][0])
    assert np.array_equal(u, g[f"p1_{form}_U"])


@pytest.mark.skipif(O.ref_tt() is None, reason="reference transient build absent")
@pytest.mark.parametrize("cau,hs,angle", [(2, 0, 10.0), (2, 2, 135.0), (3, 0, 250.0), (3, 1, 320.0)])
def test_predictor2_option_matrix_against_reference(cau, hs, angle):
    """Predictor2 over the DD shock captures and h_shock options at several
    flow angles: the whole Predictor_New loop bit-identical with the
    reference's (final state, GMRES iterations)."""
    p = G.transport_problem(13, angle_deg=angle, k=1e-3, gamma=0.1, f=0.3, cau=cau)
    p.form, p.h_shock = 1, hs
    to = O.TimeOpts(1, 3, 1e-4, 0, 3 * 0.03 + 1e-12, 1e-6, 0, 0)
    U0, its0 = O.ref_tt_predictor2(p, 0.5, 0.03, to, tol=1e-10)
    U1, a1, uB1, aB1, st = O.tt_predictor2(p, 0.5, 0.03, to, tol=1e-10)
    assert st["gmres_iterations"] == its0 and np.array_equal(U0, U1)


@pytest.mark.skipif(O.ref_tt() is None, reason="reference transient build absent")
@pytest.mark.parametrize("form,cau,hs", [(0, 1, 1), (0, 3, 2), (1, 3, 0)])
def test_predictor1_option_matrix_against_reference(form, cau, hs):
    """Predictor_Old over the SUPG / DD forms with CAU, YZBeta and CAUDD and
    the h_shock options: bit-identical with the reference's loop."""
    p = G.transport_problem(13, angle_deg=75.0, k=1e-3, gamma=0.1, f=0.3, cau=cau)
    p.form, p.h_shock = form, hs
    to = O.TimeOpts(1, 3, 1e-4, 0, 3 * 0.03 + 1e-12, 1e-6, 0, 0)
    U0, its0 = O.ref_tt_predictor1(p, 0.5, 0.03, to, tol=1e-10)
    U1, a1, st = O.tt_predictor(p, 0.5, 0.03, to, tol=1e-10)
    assert st["gmres_iterations"] == its0 and np.array_equal(U0, U1)
