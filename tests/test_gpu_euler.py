"""Compressible Euler on the GPU against the oracle (pinned bit-exactly to the
reference's Euler driver by tests/test_oracle_euler.py) and against the golden
fixtures generated from the reference itself.

The element build (12x12 Me + alpha dt Ke and residual, FP64, no FMA
contraction), the reference's 4x4 BlockDiag set-up and the residual gather
are bit-exact.  The Predictor_Old loop solves every correction to tol 1e-10
with CGS2 GMRES instead of MGS, so the state after a few steps agrees to a
relative 1e-8 with the same number of steps and corrections."""
import glob
import os

import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "eu_*.npz")))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def fg():
    from parallel_fem_codes_gb300 import femgpu
    femgpu.lib()
    return femgpu


def _perturbed(p, seed):
    rng = np.random.default_rng(seed)
    u = p.initial_state() * (1.0 + 0.05 * rng.standard_normal(p.mesh.neq))
    du = 0.01 * rng.standard_normal(p.mesh.neq)
    return u, du


@pytest.mark.parametrize("n,dimless", [(9, True), (17, True), (12, False), (33, True)])
def test_euler_assembly_bit_exact(fg, n, dimless):
    p = G.obliquo_problem(n, dimensionless=dimless)
    u, du = _perturbed(p, n)
    A, R = O.build_euler(p, u, du)
    s = fg.euler_system(p)
    Rg = s.euler_assemble(p, u, du)
    assert np.array_equal(Rg, R)
    assert np.array_equal(s.get_blocks(), A)
    # the first build of a run: initial state, du = 0
    A0, R0 = O.build_euler(p)
    assert np.array_equal(s.euler_assemble(p, p.initial_state()), R0)
    assert np.array_equal(s.get_blocks(), A0)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_euler_golden(fg, path):
    from test_oracle_euler import problem_from
    g = dict(np.load(path))
    p = problem_from(g)
    s = fg.euler_system(p)
    R = s.euler_assemble(p, g["u"], g["du"])
    assert np.array_equal(R, g["R"])
    assert np.array_equal(s.get_blocks(), g["A"])
    Rp = s.precond_setup(fg.FG_PRECOND_BLOCKDIAG, fg.FG_SETUP_REF_QUIRKS, R)
    assert np.array_equal(Rp, g["Rp"])
    assert rel(s.matvec(g["P"])[:-1], g["Q"][:-1]) < 1e-14


@pytest.mark.parametrize("stop_by_norm", [0, 1])
def test_euler_predictor(fg, stop_by_norm):
    p = G.obliquo_problem(17)
    to_o = O.TimeOpts(stop_by_norm, 2 if not stop_by_norm else 6, 1e-3, 0, 5 * p.dt, 1e-6, 0)
    uo, ao, sto = O.euler_predictor(p, to_o, tol=1e-10, kmax=25)
    s = fg.euler_system(p)
    to = fg.time_opts(stop_by_norm, to_o.max_corrections, 1e-3, 0, 5 * p.dt, 1e-6)
    ug, ag, st = s.euler_predictor(p, to, kmax=25, tol=1e-10)
    assert st["steps"] == sto["steps"] == 5
    assert abs(st["corrections"] - sto["corrections"]) <= 1
    assert rel(ug, uo) < 1e-8
    assert rel(ag, ao) < 1e-6


def test_euler_predictor_steady_state(fg):
    p = G.obliquo_problem(9, dimensionless=False)
    to_o = O.TimeOpts(1, 4, 1e-2, 1, 40 * p.dt, 1e-2, 0)
    uo, ao, sto = O.euler_predictor(p, to_o, tol=1e-10, kmax=25)
    s = fg.euler_system(p)
    ug, ag, st = s.euler_predictor(p, fg.time_opts(1, 4, 1e-2, 1, 40 * p.dt, 1e-2), kmax=25, tol=1e-10)
    assert st["steps"] == sto["steps"]
    assert rel(ug, uo) < 1e-7


def test_euler_predictor_mixed(fg):
    p = G.obliquo_problem(17)
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt, 1e-6, 0)
    uo, ao, sto = O.euler_predictor(p, to_o, tol=1e-10, kmax=25)
    s = fg.euler_system(p)
    ug, ag, st = s.euler_predictor(p, fg.time_opts(0, 2, 1e-3, 0, 3 * p.dt, 1e-6), kmax=25, tol=1e-10,
                                   precision=fg.FG_PREC_MIXED)
    assert st["steps"] == 3 and st["true_rel_residual"] <= 1e-10
    assert rel(ug, uo) < 1e-7


@pytest.mark.parametrize("precond", ["ilu0", "spike"])
@pytest.mark.parametrize("precision", [64, 32])
def test_euler_predictor_csr_rcm(fg, precond, precision):
    """The CSR operator on the RCM numbering with ILU(0) (the reference's
    "CSR" + "ILU0" configuration) or SPIKE inside the time loop reaches the
    same states as the oracle's BlockDiag run."""
    p = G.obliquo_problem(17)
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt, 1e-6, 0)
    uo, ao, sto = O.euler_predictor(p, to_o, tol=1e-10, kmax=25)
    s = fg.euler_system(p, reorder=True)
    s.set_operator(fg.FG_OP_CSR)
    kind = fg.FG_PRECOND_ILU0 if precond == "ilu0" else fg.FG_PRECOND_SPIKE
    if precond == "spike":
        s.set_spike(16, 4)
    to = fg.time_opts(0, 2, 1e-3, 0, 3 * p.dt, 1e-6, precond=kind, setup_flags=0)
    ug, ag, st = s.euler_predictor(p, to, kmax=25, tol=1e-10, precision=precision)
    assert st["steps"] == 3 and st["true_rel_residual"] <= 1e-9
    assert rel(ug, uo) < 1e-7


def test_euler_rejects_wrong_ndof(fg):
    p = G.transport_problem(9)
    s = fg.System(p.mesh)
    with pytest.raises(fg.FemGpuError):
        s.euler_set_geometry(G.obliquo_problem(9))


@pytest.mark.parametrize("scheme", [1, 2], ids=["bdf", "trbdf2"])
@pytest.mark.parametrize("steady", [0, 1])
def test_euler_time_schemes(fg, scheme, steady):
    """Predictor_Old_BDF and the TR-BDF2 loop on the device against the
    oracle (itself bit-exact with the reference's loops)."""
    p = G.obliquo_problem(17, dimensionless=not steady)
    args = (1, 4, 1e-2, 1, 40 * p.dt, 1e-2) if steady else (0, 2, 1e-3, 0, 4 * p.dt, 1e-6)
    to_o = O.TimeOpts(*args, 0, scheme)
    uo, ao, sto = O.euler_predictor(p, to_o, tol=1e-10, kmax=25)
    s = fg.euler_system(p)
    ug, ag, st = s.euler_predictor(p, fg.time_opts(*args, scheme=scheme), kmax=25, tol=1e-10)
    assert st["steps"] == sto["steps"]
    assert st["t"] == sto["t"]
    assert rel(ug, uo) < 1e-7


@pytest.mark.parametrize("dimensionless", [True, False])
def test_euler_dd_assembly_bit_exact(fg, dimensionless):
    """Build_M_K_F_DD_Transiente on the device (first build of a fresh
    system: zero element state) against the oracle, both Jacobian forms."""
    p = G.obliquo_problem(17, dimensionless=dimensionless)
    p.form = fg.FG_EULER_DD
    rng = np.random.default_rng(5)
    u = p.initial_state() * (1.0 + 0.05 * rng.standard_normal(p.mesh.neq))
    du = 0.01 * rng.standard_normal(p.mesh.neq)
    A0, R0 = O.build_euler(p, u, du)
    s = fg.euler_system(p)
    R = s.euler_assemble(p, u, du)
    assert np.array_equal(R, R0)
    assert np.array_equal(s.get_blocks(), A0)


def test_euler_dd_predictor(fg):
    """The DD loop (element state kept on the device across corrections and
    steps) against the oracle."""
    p = G.obliquo_problem(17)
    p.form = fg.FG_EULER_DD
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 4 * p.dt, 1e-6, 0)
    uo, ao, sto = O.euler_predictor(p, to_o, tol=1e-10, kmax=25)
    s = fg.euler_system(p)
    ug, ag, st = s.euler_predictor(p, fg.time_opts(0, 2, 1e-3, 0, 4 * p.dt, 1e-6), kmax=25, tol=1e-10)
    assert st["steps"] == sto["steps"] == 4
    assert rel(ug, uo) < 1e-7


# ---- "Predictor2" (DD, YZBeta): Build_M_F_DD_Transiente, calculate_DaB and
# Predictor_New with four bubble unknowns per element ----

def _p2_problem(n, dimensionless=True):
    p = G.obliquo_problem(n, dimensionless=dimensionless)
    p.form = 1
    p.invY = np.array([1.0, 0.5, 2.0, 0.25])
    return p


@pytest.mark.parametrize("n,dimless", [(9, True), (17, False), (33, True)])
def test_euler_predictor2_build_bit_exact(fg, n, dimless):
    """Me, the load, the condensation data (invN2, R2, M2) and
    calculate_DaB's increments bit-identical with the oracle (itself
    bit-identical with the reference's functions)."""
    p = _p2_problem(n, dimless)
    m = p.mesh
    rng = np.random.default_rng(n)
    u = p.initial_state() * (1 + 0.05 * rng.standard_normal(m.neq))
    du = 0.1 * rng.standard_normal(m.neq)
    uB, duB = 0.01 * rng.standard_normal(4 * m.nel), 0.01 * rng.standard_normal(4 * m.nel)
    A0, F0, c0 = O.build_euler_mfdd(p, u, du, uB, duB)
    s = fg.euler_system(p)
    F, cond = s.euler_bubble_assemble(p, u, du, uB, duB)
    assert np.array_equal(F[:-1], F0[:-1]) and F[-1] == 0.0
    assert np.array_equal(cond, c0)
    assert np.array_equal(s.get_blocks(), A0)
    Da = np.append(rng.standard_normal(m.neq), 0.0)
    assert np.array_equal(s.bubble_dab(Da), O.euler_dab(O.fill_lm(m), c0, Da))


def test_euler_predictor2_loop(fg):
    """The Predictor_New loop on the device (state, four bubble unknowns per
    element and the relaxed YZBeta state resident) against the oracle's: u
    and uB to rel-L2 1e-7, same steps and corrections."""
    p = _p2_problem(17)
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 4 * p.dt + 1e-12, 1e-6, 0, 3)
    uo, ao, uBo, aBo, sto = O.euler_predictor2(p, to_o, tol=1e-10, kmax=25)
    s = fg.euler_system(p)
    to = fg.time_opts(0, 2, 1e-3, 0, 4 * p.dt + 1e-12, 1e-6, scheme=fg.FG_TIME_PREDICTOR2)
    ug, ag, st = s.euler_predictor(p, to, kmax=25, tol=1e-10)
    uB, aB = s.bubble_state()
    assert st["steps"] == sto["steps"] == 4
    assert st["corrections"] == sto["corrections"]
    assert rel(ug, uo) < 1e-7 and rel(uB, uBo) < 1e-7
    assert rel(aB, aBo) < 1e-5


def test_euler_predictor2_needs_dd(fg):
    p = G.obliquo_problem(9)
    s = fg.euler_system(p)
    with pytest.raises(fg.FemGpuError) as e:
        s.euler_predictor(p, fg.time_opts(0, 1, 1e-3, 0, p.dt, 1e-6, max_steps=1, scheme=fg.FG_TIME_PREDICTOR2))
    assert e.value.code == fg.FG_ERR_UNSUPPORTED


# ---- ShockCapture "YZBeta" (Delta_YZBeta with invY) in the SUPG and DD builds ----

@pytest.mark.parametrize("form,dimless", [(0, True), (0, False), (1, True), (1, False)],
                         ids=["supg", "supg-dimensional", "dd", "dd-dimensional"])
def test_euler_yzbeta_assembly_bit_exact(fg, form, dimless):
    p = G.obliquo_problem(17, dimensionless=dimless)
    p.form, p.shock, p.invY = form, fg.FG_SHOCK_YZBETA, np.array([0.8, 1.5, 0.7, 0.3])
    u, du = _perturbed(p, 21 + form)
    A0, R0 = O.build_euler(p, u, du)
    s = fg.euler_system(p)
    R = s.euler_assemble(p, u, du)
    assert np.array_equal(R, R0)
    assert np.array_equal(s.get_blocks(), A0)


@pytest.mark.parametrize("form", [0, 1], ids=["supg", "dd"])
def test_euler_yzbeta_predictor(fg, form):
    p = G.obliquo_problem(17)
    p.form, p.shock, p.invY = form, fg.FG_SHOCK_YZBETA, np.array([1.0, 0.5, 2.0, 0.25])
    to_o = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt + 1e-12, 1e-6, 0)
    uo, ao, sto = O.euler_predictor(p, to_o, tol=1e-10, kmax=25)
    s = fg.euler_system(p)
    ug, ag, st = s.euler_predictor(p, fg.time_opts(0, 2, 1e-3, 0, 3 * p.dt + 1e-12, 1e-6), kmax=25, tol=1e-10)
    assert st["steps"] == sto["steps"] == 3
    assert st["corrections"] == sto["corrections"]
    assert rel(ug, uo) < 1e-7


@pytest.mark.parametrize("scheme,steady", [(4, 0), (4, 1), (5, 0)], ids=["bdf", "bdf-steady", "trbdf2"])
def test_euler_predictor2_bdf_trbdf2(fg, scheme, steady):
    """"Predictor2_BDF" (Predictor_New_BDF) and "Predictor2_TRBDF2"
    (Predictor_New_TRBDF2 with the bubble build: uB from the initial
    state's element centroids) on the device against the oracle."""
    p = _p2_problem(17)
    p.form = 1
    o_scheme = {4: 4, 5: 2}[scheme]
    to_o = O.TimeOpts(0, 2, 1e-3, steady, 3 * p.dt + 1e-12, 1e-6, 0, o_scheme)
    uo, ao, uBo, aBo, sto = O.euler_predictor2(p, to_o, tol=1e-10, kmax=25)
    s = fg.euler_system(p)
    to = fg.time_opts(0, 2, 1e-3, steady, 3 * p.dt + 1e-12, 1e-6, scheme=scheme)
    ug, ag, st = s.euler_predictor(p, to, kmax=25, tol=1e-10)
    uB, aB = s.bubble_state()
    assert st["steps"] == sto["steps"] and st["t"] == sto["t"]
    assert st["corrections"] == sto["corrections"]
    assert rel(ug, uo) < 1e-7 and rel(uB, uBo) < 1e-7


def test_euler_dd_trbdf2_is_predictor2(fg):
    """The Predictor1 DD build with TR-BDF2 is refused (the reference pairs
    it with Predictor_Old_TRBDF2, which is not restated)."""
    p = G.obliquo_problem(9)
    p.form = fg.FG_EULER_DD
    s = fg.euler_system(p)
    with pytest.raises(fg.FemGpuError) as e:
        s.euler_predictor(p, fg.time_opts(0, 1, 1e-3, 0, p.dt, 1e-6, max_steps=1, scheme=fg.FG_TIME_TRBDF2))
    assert e.value.code == fg.FG_ERR_UNSUPPORTED
