"""GPU parity of the core kernels against the oracle (CPU restatement).

Tolerances: integer/index work and the FMA-free set-up kernels (assembly,
Diag, block inverses) are bit-exact; the matvec sums per colour instead of
in element order (relative 1e-14 in FP64, 1e-6 in FP32); solutions of the
FP64 GMRES match the reference method to rel-L2 <= 1e-9 at tol 1e-10.
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


@pytest.mark.parametrize("n", [5, 17, 66])
def test_matvec_s3(fg, n):
    p = G.transport_problem(n)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    s = fg.System(m)
    s.set_blocks(A)
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    P = np.random.default_rng(n).standard_normal(m.neq + 1)
    P[-1] = 0
    Q0 = O.ebemv3_perm(lm, A, perm, inv, P)
    Q = s.matvec(P)
    assert Q[-1] == 0.0
    assert rel(Q[:-1], Q0[:-1]) < 1e-14
    Q32 = s.matvec(P, precision=32)
    assert rel(Q32[:-1], Q0[:-1]) < 1e-5
    assert np.array_equal(s.get_blocks(), A)


@pytest.mark.parametrize("ndof", [2, 3, 4])
def test_matvec_multidof(fg, ndof):
    m = G.multi_dof_mesh(9, ndof, seed=ndof)
    S = 3 * ndof
    A = G.random_blocks(m.nel, S, seed=ndof)
    s = fg.System(m)
    s.set_blocks(A)
    lm = O.fill_lm(m)
    P = np.random.default_rng(ndof).standard_normal(m.neq + 1)
    P[-1] = 0
    Q0 = O.ebemv(lm, A, m.neq, P)
    assert rel(s.matvec(P)[:-1], Q0[:-1]) < 1e-14
    assert rel(s.matvec(P, 32)[:-1], Q0[:-1]) < 1e-5


def test_assembly_bit_exact(fg):
    p = G.transport_problem(33)
    m = p.mesh
    s = fg.transport_system(p)
    for u in (None, np.random.default_rng(3).random(m.neq)):
        A0, F0 = O.build_k_f_supg(p, u)
        F = s.transport_assemble(p, u)
        assert np.array_equal(s.get_blocks(), A0)
        assert np.array_equal(F[:-1], F0[:-1])
        assert F[-1] == 0.0


def test_diag_setup_bit_exact(fg):
    p = G.transport_problem(33)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    s = fg.System(m)
    s.set_blocks(A)
    Fp = s.precond_setup(fg.FG_PRECOND_DIAG, 0, F)
    D0, inv0, Fp0 = O.diag_setup(lm, A, m.neq, F)
    assert np.array_equal(s.diag()[:-1], D0[:-1])
    assert np.array_equal(Fp[:-1], Fp0[:-1])
    # accumulation across set-ups, as the reference's Diag
    Fp2 = s.precond_setup(fg.FG_PRECOND_DIAG, fg.FG_SETUP_ACCUMULATE, F)
    D1, inv1, Fp1 = O.diag_setup(lm, A, m.neq, F, Diag=D0.copy())
    assert np.array_equal(s.diag()[:-1], D1[:-1])
    assert np.array_equal(Fp2[:-1], Fp1[:-1])
    z = s.precond_apply(F)
    assert np.array_equal(z[:-1], (F * inv1)[:-1])


@pytest.mark.parametrize("ndof", [3, 4])
def test_blockdiag_bit_exact(fg, ndof):
    m = G.multi_dof_mesh(9, ndof, seed=10 + ndof)
    A = G.random_blocks(m.nel, 3 * ndof, seed=ndof)
    F = np.random.default_rng(1).standard_normal(m.neq + 1)
    F[-1] = 0
    s = fg.System(m)
    s.set_blocks(A)
    Fp = s.precond_setup(fg.FG_PRECOND_BLOCKDIAG, fg.FG_SETUP_REF_QUIRKS, F)
    bd, ibd, Id, Fp0 = O.blockdiag_setup(m, A, F, ref_quirks=True)
    assert np.array_equal(Fp[:-1], Fp0[:-1])
    p = np.random.default_rng(2).standard_normal(m.neq + 1)
    p[-1] = 0
    assert np.array_equal(s.precond_apply(p)[:-1], O.blockdiag_apply(m, ibd, Id, p)[:-1])


@pytest.mark.parametrize("n", [17, 65])
def test_gmres_fp64_matches_reference_method(fg, n):
    p = G.transport_problem(n)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    X0, it0, _, _, Fp0 = O.ebe_diag_solve(lm, A, m.neq, F, perm, inv, kmax=30, lmax=1000, tol=1e-10)
    s = fg.System(m)
    s.set_blocks(A)
    Fp = s.precond_setup(fg.FG_PRECOND_DIAG, 0, F)
    r = s.solve(Fp, kmax=30, lmax=1000, tol=1e-10, F_true=F)
    assert r.stats["converged"] == 1 and r.stats["status"] == 0
    assert abs(r.stats["iterations"] - it0) <= max(2, it0 // 50)
    assert rel(r.x[:-1], X0[:-1]) <= 1e-9
    res = np.linalg.norm(F[:-1] - O.ebemv3_perm(lm, A, perm, inv, r.x)[:-1]) / np.linalg.norm(F[:-1])
    assert abs(res - r.stats["true_rel_residual"]) <= 1e-3 * res + 1e-15


@pytest.mark.parametrize("n", [17, 65])
def test_gmres_mixed_reaches_true_residual(fg, n):
    p = G.transport_problem(n)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    s = fg.System(m)
    s.set_blocks(A)
    Fp = s.precond_setup(fg.FG_PRECOND_DIAG, 0, F)
    r64 = s.solve(Fp, tol=1e-10, F_true=F)
    r32 = s.solve(Fp, tol=1e-10, F_true=F, precision=fg.FG_PREC_MIXED)
    assert r32.stats["converged"] == 1
    res = np.linalg.norm(F[:-1] - O.ebemv3_perm(lm, A, perm, inv, r32.x)[:-1]) / np.linalg.norm(F[:-1])
    assert res <= 1e-10
    assert r32.stats["true_rel_residual"] <= 1e-10
    assert rel(r32.x[:-1], r64.x[:-1]) <= 1e-6


def test_transport_process_matches_oracle(fg):
    p = G.transport_problem(33)
    U0, nl0, it0 = O.transport_process(p, 1e-10, 1e-3, 30, 1000)
    s = fg.transport_system(p)
    U, st = s.transport_process(p, 30, 1000, 1e-10, 1e-3)
    assert st["nonlinear_iterations"] == nl0
    assert rel(U, U0) <= 1e-9


def test_teste_exact_solution(fg):
    """TESTE problem: k = 1, beta = 0, f = 0, u = 10 on the boundary -> u = 10."""
    p = G.transport_problem(17, angle_deg=0.0, k=1.0, upmode=1, upval=10.0)
    p.beta = (0.0, 0.0)
    s = fg.transport_system(p)
    U, st = s.transport_process(p, 30, 1000, 1e-12, 1e-6)
    assert np.max(np.abs(U - 10.0)) < 1e-9


@pytest.mark.parametrize("shock", [1, 2], ids=["cau", "caudd"])
def test_dd_assembly_bit_exact(fg, shock):
    """Build_K_F_DD (StabilizationForm "DD") on the device against the
    oracle, which is bit-exact with the reference's build."""
    p = G.transport_problem(33, angle_deg=110.0, k=1e-4, gamma=0.2, f=0.5, cau=shock)
    p.form = fg.FG_TRANSPORT_DD
    m = p.mesh
    s = fg.transport_system(p)
    for u in (None, np.random.default_rng(5).random(m.neq)):
        A0, F0 = O.build_k_f_supg(p, u)
        F = s.transport_assemble(p, u)
        assert np.array_equal(s.get_blocks(), A0)
        assert np.array_equal(F[:-1], F0[:-1])


def test_dd_process_matches_oracle(fg):
    p = G.transport_problem(33, cau=2)
    p.form = fg.FG_TRANSPORT_DD
    U0, nl0, it0 = O.transport_process(p, 1e-10, 1e-3, 30, 1000)
    s = fg.transport_system(p)
    U, st = s.transport_process(p, 30, 1000, 1e-10, 1e-3)
    assert st["nonlinear_iterations"] == nl0
    assert rel(U, U0) <= 1e-9


def test_caudd_needs_dd_form(fg):
    p = G.transport_problem(9, cau=2)
    s = fg.transport_system(p)
    with pytest.raises(Exception):
        s.transport_assemble(p)


@pytest.mark.parametrize("form,shock,hs", [(0, 3, 0), (0, 1, 1), (0, 3, 2), (1, 3, 1), (1, 2, 2)])
def test_shock_options_device(fg, form, shock, hs):
    """YZBeta (state on the device) and the h_shock options: the first build
    of a fresh system and the whole Process loop against the oracle."""
    p = G.transport_problem(33, angle_deg=110.0, k=1e-4, gamma=0.2, f=0.5, cau=shock)
    p.form, p.h_shock = form, hs
    u = np.random.default_rng(11).random(p.mesh.neq)
    A0, F0 = O.build_k_f_supg(p, u)
    s = fg.transport_system(p)
    F = s.transport_assemble(p, u)
    assert np.array_equal(s.get_blocks(), A0) and np.array_equal(F[:-1], F0[:-1])
    U0, nl0, it0 = O.transport_process(p, 1e-10, 1e-3, 30, 1000)
    U, st = s.transport_process(p, 30, 1000, 1e-10, 1e-3)
    assert st["nonlinear_iterations"] == nl0
    assert rel(U, U0) <= 1e-9
