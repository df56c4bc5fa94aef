"""The Euler oracle (oracle/euler.c) against the golden fixtures generated
from the reference's own C (03_Euler_Equations driver: Fill_LM,
Build_M_K_F_SUPG with Delta_CAU and both Jacobian forms,
BlockDiag_precond_EBE_setup, ebemvNDOF4, Predictor_Old with the Criteria.c
stop tests), and against the reference build itself where it is present.
Everything is bit-exact, including the time loop."""
import glob
import os

import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "eu_*.npz")))


def problem_from(g):
    m = G.Mesh(g["x"], g["y"], g["ien"], 4, g["type"], g["invp"], int(g["neq"]))
    gm, mach, dl, tol, alpha, dt = [float(v) for v in g["params"]]
    return G.euler_problem(m, gm, mach, bool(dl), tol, alpha, dt, g["coef"], bool(g["wall"]), g["init"])


def topts_from(g):
    a = g["topts"]
    return O.TimeOpts(int(a[0]), int(a[1]), float(a[2]), int(a[3]), float(a[4]), float(a[5]), 0)


@pytest.fixture(scope="module", params=GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def case(request, oracle_lib):
    g = dict(np.load(request.param))
    return g, problem_from(g)


def test_golden_present():
    assert len(GOLDEN) >= 2


def test_fill_lm(case):
    g, p = case
    assert np.array_equal(O.fill_lm(p.mesh).reshape(-1), g["lm"].reshape(-1))


def test_build_bit_exact(case):
    g, p = case
    A, R = O.build_euler(p, g["u"], g["du"])
    assert np.array_equal(A, g["A"])
    assert np.array_equal(R, g["R"])


def test_blockdiag_4x4_bit_exact(case):
    g, p = case
    bd, ibd, Id, Rp = O.blockdiag_setup(p.mesh, g["A"], g["R"], ref_quirks=True)
    assert np.array_equal(ibd, g["inv"])
    assert np.array_equal(Rp, g["Rp"])


def test_ebemv_ndof4_bit_exact(case):
    g, p = case
    Q = O.ebemv(O.fill_lm(p.mesh), g["A"], p.mesh.neq, g["P"])
    assert np.array_equal(Q, g["Q"])


def test_predictor_bit_exact(case):
    g, p = case
    u, a, st = O.euler_predictor(p, topts_from(g), tol=1e-10, kmax=25, lmax=1000)
    assert st["gmres_iterations"] == int(g["gmres_its"])
    assert st["t"] == float(g["t"])
    assert np.array_equal(u, g["U"])


SCHEMES = os.path.join(os.path.dirname(__file__), "golden", "time_schemes_euler.npz")


@pytest.mark.parametrize("name", ["eu_9_obliquo", "eu_7_dimensional"])
@pytest.mark.parametrize("scheme", [1, 2], ids=["bdf", "trbdf2"])
def test_time_schemes_bit_exact(name, scheme, oracle_lib):
    """Predictor_Old_BDF and (bubble-free) Predictor_New_TRBDF2 against the
    reference's own loops run by the golden generator."""
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz")))
    p = problem_from(g)
    gs = np.load(SCHEMES)
    to = topts_from(g)
    to.scheme = scheme
    u, a, st = O.euler_predictor(p, to, tol=1e-10, kmax=25, lmax=1000)
    key = f"{name}_s{scheme}"
    assert st["gmres_iterations"] == int(gs[key + "_its"])
    assert st["t"] == float(gs[key + "_t"])
    assert np.array_equal(u, gs[key + "_U"])


@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_time_schemes_against_reference_build(scheme, oracle_lib):
    """The same against the reference build itself, on a third case, where
    the reference sources were compiled (oracle/_ref)."""
    if O.ref_euler() is None:
        pytest.skip("reference build (oracle/_ref) not present")
    p = G.obliquo_problem(11)
    to = O.TimeOpts(1, 3, 1e-2, 0, 3 * p.dt, 1e-6, 0, scheme)
    U, its, t = O.ref_euler_predictor(p, to, 1e-10, 25, 1000)
    u, a, st = O.euler_predictor(p, to, tol=1e-10, kmax=25, lmax=1000)
    assert st["gmres_iterations"] == its and st["t"] == t
    assert np.array_equal(u, U)


def test_obliquo_layout():
    p = G.obliquo_problem(9)
    m = p.mesh
    t = m.type.reshape(-1, 4)
    bottom = np.abs(m.y) <= 1e-15
    inflow = ((np.abs(m.x) <= 1e-15) | (np.abs(m.y - 1.0) <= 1e-15)) & ~bottom
    assert np.all(t[bottom] == [1, 1, 0, 1])
    assert np.all(t[inflow] == 0)
    assert np.all(t[~bottom & ~inflow] == 1)
    up = p.upresc.reshape(-1, 4)
    assert np.all(up[bottom & (m.x > 0), 2] == 0.0)
    assert up[0, 2] == -0.17365                       # the corner keeps the inflow value
    assert np.array_equal(p.initial_state()[m.invp.reshape(-1, 4)[t[:, 0] != 0, 0]], np.ones(int((t[:, 0] != 0).sum())))


@pytest.mark.skipif(O.ref_euler() is None, reason="reference build absent (oracle/_ref)")
@pytest.mark.parametrize("n,dimless", [(15, True), (10, False)])
def test_against_reference_build(n, dimless):
    p = G.obliquo_problem(n, dimensionless=dimless)
    rng = np.random.default_rng(n)
    u = p.initial_state() * (1.0 + 0.1 * rng.standard_normal(p.mesh.neq))
    du = 0.05 * rng.standard_normal(p.mesh.neq)
    A, R = O.build_euler(p, u, du)
    Ar, Rr = O.ref_euler_build(p, u, du)
    assert np.array_equal(A, Ar) and np.array_equal(R, Rr)


DDE = os.path.join(os.path.dirname(__file__), "golden", "dd_euler.npz")


@pytest.mark.parametrize("name", ["eu_9_obliquo", "eu_7_dimensional"])
def test_dd_bit_exact(name, oracle_lib):
    """StabilizationForm "DD" (Build_M_K_F_DD_Transiente with Delta_DD):
    blocks and residual at a state, and the Predictor_Old loop with its
    element state (bubbles, relaxed delta), against the reference's own."""
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz")))
    p = problem_from(g)
    p.form = 1
    d = np.load(DDE)
    A, R = O.build_euler(p, d[name + "_u"], d[name + "_du"])
    assert np.array_equal(A, d[name + "_A"]) and np.array_equal(R, d[name + "_R"])
    u, a, st = O.euler_predictor(p, topts_from(g), tol=1e-10, kmax=25, lmax=1000)
    assert st["gmres_iterations"] == int(d[name + "_its"]) and st["t"] == float(d[name + "_t"])
    assert np.array_equal(u, d[name + "_U"])


def test_dd_against_reference_build(oracle_lib):
    if O.ref_euler() is None:
        pytest.skip("reference build (oracle/_ref) not present")
    p = G.obliquo_problem(11)
    p.form = 1
    rng = np.random.default_rng(11)
    u = p.initial_state() * (1.0 + 0.05 * rng.standard_normal(p.mesh.neq))
    du = 0.01 * rng.standard_normal(p.mesh.neq)
    A0, R0 = O.ref_euler_build(p, u, du)
    A1, R1 = O.build_euler(p, u, du)
    assert np.array_equal(A0, A1) and np.array_equal(R0, R1)


def test_block_scaling_against_reference(oracle_lib):
    """Block_scaling_EBE restated (oracle/ebe_gmres.c) against the reference's
    function called directly (the Euler driver installs it, never calls it)."""
    if O.ref_euler() is None:
        pytest.skip("reference build (oracle/_ref) not present")
    for p in (G.obliquo_problem(9), G.obliquo_problem(7, dimensionless=False)):
        m = p.mesh
        u = p.initial_state() * (1.0 + 0.05 * np.random.default_rng(2).standard_normal(m.neq))
        A, R = O.build_euler(p, u)
        A1, F1, inv1 = O.ref_euler_block_scale(m, A, R)
        bd, ibd, Id, Fo = O.blockdiag_setup(m, A, R, ref_quirks=True)
        assert np.array_equal(inv1, ibd) and np.array_equal(F1, Fo)
        assert np.array_equal(A1, O.block_scale(m, A, ibd))


# ---- TimeIntegration "Predictor2" with "DD" and "YZBeta": Build_M_F_DD_Transiente.c,
# Delta_YZBeta.c, Delta_YZBetaNMV.c, calculate_DaB.c and Predictor_New.c ----

def _p2_problem(n=9):
    p = G.obliquo_problem(n)
    p.invY = np.array([1.0, 0.5, 2.0, 0.25])
    return p


@pytest.fixture(scope="module")
def p2gold():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "euler_predictor2_ref.npz"))


def test_predictor2_build_matches_reference_golden(p2gold):
    """Me, F, the condensation data (invN2, R2, M2) and calculate_DaB's
    bubble increments bit-identical with the reference's own functions."""
    g = p2gold
    p = _p2_problem()
    A, F, cond = O.build_euler_mfdd(p, g["u"], g["du"], g["uB"], g["duB"])
    assert np.array_equal(A, g["A"]) and np.array_equal(F, g["F"]) and np.array_equal(cond, g["cond"])
    assert np.array_equal(O.euler_dab(O.fill_lm(p.mesh), cond, g["Da"]), g["DaB"])


def test_predictor2_loop_matches_reference_golden(p2gold):
    """The whole Predictor_New loop (3 steps x 2 corrections, BlockDiag,
    GMRES): final state and GMRES iterations equal the reference's."""
    p = _p2_problem()
    to = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt + 1e-12, 1e-6, 0, 3)
    u, a, uB, aB, st = O.euler_predictor2(p, to, 1e-10, 25, 1000)
    assert st["steps"] == 3 and st["corrections"] == 6
    assert st["gmres_iterations"] == int(p2gold["its"][0])
    assert np.array_equal(u, p2gold["U"])
    assert np.abs(uB).max() > 0                      # the bubbles move


@pytest.mark.parametrize("scheme", [4, 2], ids=["predictor2_bdf", "predictor2_trbdf2"])
def test_predictor2_bdf_trbdf2_match_reference_golden(p2gold, scheme):
    """Predictor_New_BDF ("Predictor2_BDF": a BDF1 step with Alpha_Build 1,
    then BDF2 with 2/3, u_old kept per step) and Predictor_New_TRBDF2
    ("Predictor2_TRBDF2": uB from the initial state, TR and BDF2 stages on
    uB too) with Build_M_F_DD_Transiente: final state and GMRES iterations
    equal the reference's."""
    p = _p2_problem()
    to = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt + 1e-12, 1e-6, 0, scheme)
    u, a, uB, aB, st = O.euler_predictor2(p, to, 1e-10, 25, 1000)
    assert st["gmres_iterations"] == int(p2gold[f"its_s{scheme}"][0])
    assert np.array_equal(u, p2gold[f"U_s{scheme}"])


@pytest.mark.skipif(O.ref_euler() is None, reason="reference build (oracle/_ref) not present")
def test_predictor2_against_reference_build():
    p = _p2_problem(11)
    p.invY = np.array([0.8, 1.5, 0.7, 0.3])
    m = p.mesh
    rng = np.random.default_rng(5)
    u = p.initial_state() * (1 + 0.05 * rng.standard_normal(m.neq))
    du = 0.1 * rng.standard_normal(m.neq)
    uB, duB = 0.01 * rng.standard_normal(4 * m.nel), 0.01 * rng.standard_normal(4 * m.nel)
    Da = np.append(rng.standard_normal(m.neq), 1.0)
    A0, F0, c0, D0 = O.ref_euler_mfdd_build(p, u, du, uB, duB, Da)
    A1, F1, c1 = O.build_euler_mfdd(p, u, du, uB, duB)
    assert np.array_equal(A0, A1) and np.array_equal(F0, F1) and np.array_equal(c0, c1)
    assert np.array_equal(D0, O.euler_dab(O.fill_lm(m), c1, Da))
    to = O.TimeOpts(1, 3, 1e-4, 0, 2 * p.dt + 1e-12, 1e-6, 0, 3)
    U0, its0, t0 = O.ref_euler_predictor(p, to, 1e-10, 25, 1000)
    U1, a1, uB1, aB1, st = O.euler_predictor2(p, to, 1e-10, 25, 1000)
    assert st["gmres_iterations"] == its0 and np.array_equal(U0, U1)


def test_predictor2_bubble_rows_are_solved():
    """The bubble rows of each element's system, M2 . Da_e + N2 DaB = R2,
    hold for calculate_DaB's increments (static condensation is exact)."""
    p = _p2_problem()
    m = p.mesh
    rng = np.random.default_rng(9)
    A, F, cond = O.build_euler_mfdd(p, p.initial_state(), 0.1 * rng.standard_normal(m.neq),
                                    0.01 * rng.standard_normal(4 * m.nel), 0.01 * rng.standard_normal(4 * m.nel))
    lm = O.fill_lm(m)
    Da = np.append(rng.standard_normal(m.neq), 0.0)
    DaB = O.euler_dab(lm, cond, Da).reshape(m.nel, 4)
    invN2, R2, M2 = cond[:, 0], cond[:, 1:5], cond[:, 5:].reshape(m.nel, 4, 12)
    resid = np.einsum("erj,ej->er", M2, Da[lm]) + DaB / invN2[:, None] - R2
    assert np.abs(resid).max() <= 1e-12 * max(np.abs(R2).max(), 1.0)


# ---- ShockCapture "YZBeta" (Delta_YZBeta.c) in the SUPG and Predictor1 DD builds ----

@pytest.fixture(scope="module")
def yzgold():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "euler_yzbeta_ref.npz"))


def _yz_problem(form, n=9):
    p = G.obliquo_problem(n)
    p.form, p.shock, p.invY = form, 3, np.array([1.0, 0.5, 2.0, 0.25])
    return p


@pytest.mark.parametrize("form", [0, 1], ids=["supg", "dd"])
def test_yzbeta_build_matches_reference_golden(yzgold, form):
    key = f"yz_{form}"
    A, R = O.build_euler(_yz_problem(form), yzgold[key + "_u"], yzgold[key + "_du"])
    assert np.array_equal(A, yzgold[key + "_A"]) and np.array_equal(R, yzgold[key + "_R"])


@pytest.mark.parametrize("form", [0, 1], ids=["supg", "dd"])
@pytest.mark.parametrize("scheme", [0, 1], ids=["predictor", "bdf"])
def test_yzbeta_loops_match_reference_golden(yzgold, form, scheme):
    p = _yz_problem(form)
    to = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt + 1e-12, 1e-6, 0, scheme)
    u, a, st = O.euler_predictor(p, to, 1e-10, 25, 1000)
    key = f"yz_{form}_s{scheme}"
    assert st["gmres_iterations"] == int(yzgold[key + "_its"][0])
    assert np.array_equal(u, yzgold[key + "_U"])


@pytest.mark.skipif(O.ref_euler() is None, reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("form,dimless", [(0, False), (1, False), (0, True)])
def test_yzbeta_against_reference_build(form, dimless):
    p = G.obliquo_problem(11, dimensionless=dimless)
    p.form, p.shock, p.invY = form, 3, np.array([0.8, 1.5, 0.7, 0.3])
    rng = np.random.default_rng(12 + form)
    u = p.initial_state() * (1 + 0.05 * rng.standard_normal(p.mesh.neq))
    du = 0.05 * rng.standard_normal(p.mesh.neq)
    A0, R0 = O.ref_euler_build(p, u, du)
    A1, R1 = O.build_euler(p, u, du)
    assert np.array_equal(A0, A1) and np.array_equal(R0, R1)


@pytest.mark.skipif(O.ref_euler() is None, reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("scheme", [3, 4, 2], ids=["predictor2", "predictor2_bdf", "predictor2_trbdf2"])
@pytest.mark.parametrize("dimless,stop_norm", [(True, 1), (False, 0)])
def test_predictor2_schemes_against_reference_build(scheme, dimless, stop_norm):
    """Every Predictor2 loop in both Jacobian forms and both correction stop
    tests: bit-identical with the reference's Predictor_New* loops."""
    p = G.obliquo_problem(9, dimensionless=dimless)
    p.form, p.invY = 2, np.array([0.9, 0.6, 1.7, 0.4])
    to = O.TimeOpts(stop_norm, 3, 1e-4, 0, 3 * p.dt + 1e-12, 1e-6, 0, scheme)
    U0, its0, _ = O.ref_euler_predictor(p, to, 1e-10, 25, 1000)
    U1, a1, uB1, aB1, st = O.euler_predictor2(p, to, 1e-10, 25, 1000)
    assert st["gmres_iterations"] == its0 and np.array_equal(U0, U1)


@pytest.mark.skipif(O.ref_euler() is None, reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("form", [0, 1], ids=["supg", "dd"])
def test_yzbeta_steady_stop_against_reference_build(form):
    """YZBeta with the steady-state time stop (Predictor_Old)."""
    p = G.obliquo_problem(9)
    p.form, p.shock, p.invY = form, 3, np.array([1.0, 0.5, 2.0, 0.25])
    to = O.TimeOpts(1, 4, 1e-3, 1, 20 * p.dt, 1e-3, 0, 0)
    U0, its0, t0 = O.ref_euler_predictor(p, to, 1e-10, 25, 1000)
    U1, a1, st = O.euler_predictor(p, to, 1e-10, 25, 1000)
    assert np.all(np.isfinite(U0))
    assert st["gmres_iterations"] == its0 and st["t"] == t0 and np.array_equal(U0, U1)
