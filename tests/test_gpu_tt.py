"""Transient SUPG/CAU transport on the GPU (fg_tt_assemble,
fg_tt_predictor) against the CPU restatement (oracle/tt.c): blocks
Ae = me + alpha dt ke and the residual R = F - me du - ke u are
bit-identical (same terms, same element-order accumulation, no FMA
contraction); the Predictor_Old loop with accumulating Diag reaches the
oracle's states to rel-L2 1e-8 at tol 1e-10, in FP64 and mixed precision.
"Predictor2" (fg_tt_bubble_assemble, FG_TIME_PREDICTOR2): the bubble
build, its condensation data and calculate_DaB bit-identical, the loop's
u and bubble unknowns to 1e-8."""
import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    from parallel_fem_codes_gb300 import femgpu
    femgpu.lib()
    return femgpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("n,cau,reorder", [(9, True, True), (33, True, True), (33, False, False), (48, True, True)])
def test_tt_assembly_bit_exact(fg, n, cau, reorder):
    p = G.transport_problem(n, angle_deg=35.0, k=1e-3, gamma=0.2, f=0.5, cau=cau)
    rng = np.random.default_rng(n)
    u = rng.random(p.mesh.neq)
    du = rng.standard_normal(p.mesh.neq)
    A0, R0 = O.build_tt(p, 0.5, 0.05, u=u, du=du)
    s = fg.transport_system(p, reorder=reorder)
    R = s.tt_assemble(p, 0.5, 0.05, u, du)
    assert np.array_equal(R[:-1], R0[:-1]) and R[-1] == 0.0
    assert np.array_equal(s.get_blocks(), A0)


@pytest.mark.parametrize("precision", [64, 32])
def test_tt_predictor(fg, precision):
    p = G.transport_problem(33, angle_deg=30.0, k=1e-3, f=0.0)
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 10 * 0.02, 1e-6, 0)
    uo, ao, sto = O.tt_predictor(p, 0.5, 0.02, to_o, tol=1e-10, kmax=30)
    s = fg.transport_system(p)
    to = fg.time_opts(0, 2, 1e-3, 0, 10 * 0.02, 1e-6, precond=fg.FG_PRECOND_DIAG, setup_flags=0)
    ug, ag, st = s.tt_predictor(p, 0.5, 0.02, to, kmax=30, tol=1e-10, precision=precision)
    assert st["steps"] == sto["steps"] == 10
    assert st["corrections"] == sto["corrections"]
    assert rel(ug, uo) < 1e-8
    assert rel(ag, ao) < 1e-6
    if precision == 32:
        assert st["true_rel_residual"] <= 1e-10


def test_tt_predictor_steady_stop(fg):
    p = G.transport_problem(17, angle_deg=30.0, k=1e-2, cau=False)
    to_o = O.TimeOpts(1, 5, 1e-6, 1, 1e3, 1e-7, 0)
    uo, ao, sto = O.tt_predictor(p, 0.5, 0.05, to_o, tol=1e-12)
    s = fg.transport_system(p)
    ug, ag, st = s.tt_predictor(p, 0.5, 0.05, fg.time_opts(1, 5, 1e-6, 1, 1e3, 1e-7, precond=fg.FG_PRECOND_DIAG,
                                                          setup_flags=0), tol=1e-12)
    assert st["steps"] == sto["steps"]
    assert rel(ug, uo) < 1e-8


@pytest.mark.parametrize("scheme", [1, 2], ids=["bdf", "trbdf2"])
def test_tt_time_schemes(fg, scheme):
    """The BDF and TR-BDF2 loops drive the transient transport build too
    (the reference shares its predictors between the drivers)."""
    p = G.transport_problem(33, angle_deg=30.0, k=1e-3, f=0.0)
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 6 * 0.02, 1e-6, 0, scheme)
    uo, ao, sto = O.tt_predictor(p, 0.5, 0.02, to_o, tol=1e-10, kmax=30)
    s = fg.transport_system(p)
    to = fg.time_opts(0, 2, 1e-3, 0, 6 * 0.02, 1e-6, precond=fg.FG_PRECOND_DIAG, setup_flags=0, scheme=scheme)
    ug, ag, st = s.tt_predictor(p, 0.5, 0.02, to, kmax=30, tol=1e-10)
    assert st["steps"] == sto["steps"] and st["t"] == sto["t"]
    assert st["corrections"] == sto["corrections"]
    assert rel(ug, uo) < 1e-8


@pytest.mark.parametrize("cau", [0, 2], ids=["none", "caudd"])
def test_tt_dd_assembly_bit_exact(fg, cau):
    """Build_M_K_R_DD on the device (first build of a fresh system: zero
    shock-capture state) against the oracle."""
    p = G.transport_problem(33, angle_deg=110.0, k=1e-3, gamma=0.2, f=0.5, cau=cau)
    p.form = fg.FG_TRANSPORT_DD
    rng = np.random.default_rng(4)
    u = rng.random(p.mesh.neq)
    du = rng.standard_normal(p.mesh.neq)
    A0, R0 = O.build_tt(p, 0.5, 0.05, u=u, du=du)
    s = fg.transport_system(p)
    R = s.tt_assemble(p, 0.5, 0.05, u, du)
    assert np.array_equal(R[:-1], R0[:-1]) and R[-1] == 0.0
    assert np.array_equal(s.get_blocks(), A0)


def test_tt_dd_predictor(fg):
    """The Predictor_Old loop with the DD build and CAUDD (state kept on the
    device across the corrections and steps) against the oracle."""
    p = G.transport_problem(33, angle_deg=30.0, k=1e-3, f=0.0, cau=2)
    p.form = fg.FG_TRANSPORT_DD
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 8 * 0.02, 1e-6, 0)
    uo, ao, sto = O.tt_predictor(p, 0.5, 0.02, to_o, tol=1e-10, kmax=30)
    s = fg.transport_system(p)
    to = fg.time_opts(0, 2, 1e-3, 0, 8 * 0.02, 1e-6, precond=fg.FG_PRECOND_DIAG, setup_flags=0)
    ug, ag, st = s.tt_predictor(p, 0.5, 0.02, to, kmax=30, tol=1e-10)
    assert st["steps"] == sto["steps"] == 8
    assert st["corrections"] == sto["corrections"]
    assert rel(ug, uo) < 1e-8


@pytest.mark.parametrize("form,hs", [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (1, 2)],
                         ids=["supg-2sqrtA", "supg-opt1", "supg-opt2", "dd-2sqrtA", "dd-opt1", "dd-opt2"])
def test_tt_yzbeta_h_shock_bit_exact(fg, form, hs):
    """YZBeta_ShockCapture (Ru with du/dt) with each h_shock option, in the
    SUPG and the DD transient builds (DD relaxed against the element's
    previous coefficient: zero on a fresh system), against the oracle."""
    p = G.transport_problem(33, angle_deg=50.0, k=1e-3, gamma=0.2, f=0.5, cau=fg.FG_SHOCK_YZBETA)
    p.form, p.h_shock = form, hs
    rng = np.random.default_rng(11 + hs)
    u = rng.random(p.mesh.neq)
    du = rng.standard_normal(p.mesh.neq)
    A0, R0 = O.build_tt(p, 0.5, 0.05, u=u, du=du)
    s = fg.transport_system(p)
    R = s.tt_assemble(p, 0.5, 0.05, u, du)
    assert np.array_equal(R[:-1], R0[:-1]) and R[-1] == 0.0
    assert np.array_equal(s.get_blocks(), A0)


def test_tt_yzbeta_dd_predictor(fg):
    """The DD time loop with YZBeta (relaxed state on the device) against
    the oracle's."""
    p = G.transport_problem(33, angle_deg=30.0, k=1e-3, f=0.0, cau=fg.FG_SHOCK_YZBETA)
    p.form, p.h_shock = fg.FG_TRANSPORT_DD, 2
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 6 * 0.02, 1e-6, 0)
    uo, ao, sto = O.tt_predictor(p, 0.5, 0.02, to_o, tol=1e-10, kmax=30)
    s = fg.transport_system(p)
    to = fg.time_opts(0, 2, 1e-3, 0, 6 * 0.02, 1e-6, precond=fg.FG_PRECOND_DIAG, setup_flags=0)
    ug, ag, st = s.tt_predictor(p, 0.5, 0.02, to, kmax=30, tol=1e-10)
    assert st["steps"] == sto["steps"] == 6
    assert st["corrections"] == sto["corrections"]
    assert rel(ug, uo) < 1e-8


# ---- TimeIntegration "Predictor2" with the DD form (Build_M_F_DD.c,
# calculate_DaB.c, Predictor_New.c): one bubble unknown per element ----

@pytest.mark.parametrize("n,cau,hs,reorder", [(17, 2, 0, True), (33, 3, 2, True), (33, 2, 1, False)])
def test_tt_predictor2_build_bit_exact(fg, n, cau, hs, reorder):
    """Me, the load, the condensation data and calculate_DaB's increments
    bit-identical with the oracle (itself bit-identical with the
    reference's own functions, tests/test_oracle_tt.py)."""
    p = G.transport_problem(n, angle_deg=35.0, k=1e-3, gamma=0.2, f=0.5, cau=cau)
    p.form, p.h_shock = fg.FG_TRANSPORT_DD, hs
    m = p.mesh
    rng = np.random.default_rng(n + cau)
    u, du = rng.random(m.neq), rng.standard_normal(m.neq)
    uB, duB = rng.random(m.nel), rng.standard_normal(m.nel)
    A0, F0, c0 = O.build_tt_mfdd(p, 0.5, 0.05, u, du, uB, duB)
    s = fg.transport_system(p, reorder=reorder)
    F, cond = s.tt_bubble_assemble(p, 0.5, 0.05, u, du, uB, duB)
    assert np.array_equal(F[:-1], F0[:-1]) and F[-1] == 0.0
    assert np.array_equal(cond, c0)
    assert np.array_equal(s.get_blocks(), A0)
    Da = np.append(rng.standard_normal(m.neq), 0.0)
    assert np.array_equal(s.bubble_dab(Da), O.tt_dab(O.fill_lm(m), c0, Da))


@pytest.mark.parametrize("cau", [2, 3], ids=["caudd", "yzbeta"])
def test_tt_predictor2_loop(fg, cau):
    """The Predictor_New loop on the device (state, bubble unknowns and
    shock-capture state resident) against the oracle's loop: u and uB to
    rel-L2 1e-8, a and aB to 1e-6, same steps and corrections."""
    p = G.transport_problem(33, angle_deg=30.0, k=1e-3, f=0.0, cau=cau)
    p.form = fg.FG_TRANSPORT_DD
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 6 * 0.02, 1e-6, 0, 0)
    uo, ao, uBo, aBo, sto = O.tt_predictor2(p, 0.5, 0.02, to_o, tol=1e-10, kmax=30)
    s = fg.transport_system(p)
    to = fg.time_opts(0, 2, 1e-3, 0, 6 * 0.02, 1e-6, precond=fg.FG_PRECOND_DIAG, setup_flags=0,
                      scheme=fg.FG_TIME_PREDICTOR2)
    ug, ag, st = s.tt_predictor(p, 0.5, 0.02, to, kmax=30, tol=1e-10)
    uB, aB = s.bubble_state()
    assert st["steps"] == sto["steps"] == 6
    assert st["corrections"] == sto["corrections"]
    assert rel(ug, uo) < 1e-8 and rel(uB, uBo) < 1e-8
    assert rel(ag, ao) < 1e-6 and rel(aB, aBo) < 1e-6


def test_tt_predictor2_needs_dd(fg):
    """Predictor2 exists for the DD form only (setStabilizationForm.c:51-54)."""
    p = G.transport_problem(9, angle_deg=30.0, k=1e-3)
    s = fg.transport_system(p)
    to = fg.time_opts(0, 1, 1e-3, 0, 0.02, 1e-6, precond=fg.FG_PRECOND_DIAG, setup_flags=0,
                      scheme=fg.FG_TIME_PREDICTOR2)
    with pytest.raises(fg.FemGpuError) as e:
        s.tt_predictor(p, 0.5, 0.02, to)
    assert e.value.code == fg.FG_ERR_UNSUPPORTED
    p.form = fg.FG_TRANSPORT_DD                     # _BDF / _TRBDF2: Euler driver only
    for scheme in (fg.FG_TIME_PREDICTOR2_BDF, fg.FG_TIME_PREDICTOR2_TRBDF2):
        to.scheme = scheme
        with pytest.raises(fg.FemGpuError) as e:
            s.tt_predictor(p, 0.5, 0.02, to)
        assert e.value.code == fg.FG_ERR_UNSUPPORTED
