"""The element preconditioners of the steady driver (Preconditioner "LUe"
and "SGSe"; 00_CommonFiles/Solvers_and_Preconditioners/EBE/LU_precond_EBE.c,
LU_precond_EBE_setup.c, SGS_precond_EBE.c, SGS_precond_EBE_setup.c, with
pgmres.c applying precondR to v before each matvec and to X at the end).

The oracle's restatement (oracle/ebe_gmres.c: or_lue_setup, or_lue_apply,
or_sgs_fwd, or_sgs_bwd, or_ebe_elem_solve) is pinned bit for bit to the
reference's own functions: tests/golden/elem_prec_sst.npz holds one
application of each sweep and the set-up + pgmres solve of each
preconditioner, made by the reference build (oracle/_ref/libref_sst.so)."""
import os

import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

GOLD = os.path.join(os.path.dirname(__file__), "golden", "elem_prec_sst.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _problem(n):
    p = G.transport_problem(n, angle_deg=30.0, k=1e-3)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    return m, A, F, lm, perm, inv


@pytest.mark.parametrize("n", [17, 33])
@pytest.mark.parametrize("kind", [1, 2, 3])
def test_sweeps_match_reference(gold, n, kind):
    m, A, F, lm, perm, inv = _problem(n)
    z = gold[f"ep_{n}_z"]
    out = O.elem_prec_apply(kind, lm, A, m.neq, z)
    assert np.array_equal(out, gold[f"ep_{n}_apply{kind}"])
    assert out[m.neq] == 0.0


@pytest.mark.parametrize("n", [17, 33])
@pytest.mark.parametrize("kind", [1, 2])
def test_solves_match_reference(gold, n, kind):
    m, A, F, lm, perm, inv = _problem(n)
    X, it, Fp = O.ebe_elem_solve(kind, lm, A, m.neq, F, perm, inv, kmax=30, lmax=200, tol=1e-10)
    assert it == int(gold[f"ep_{n}_it{kind}"][0])
    assert np.array_equal(Fp[:-1], gold[f"ep_{n}_F{kind}"][:-1])
    assert np.array_equal(X[:-1], gold[f"ep_{n}_X{kind}"][:-1])


def test_solution_solves_the_system():
    """The SGSe solve returns R X (the right preconditioner applied at the
    end): A x = F to the tolerance."""
    m, A, F, lm, perm, inv = _problem(17)
    X, it, _ = O.ebe_elem_solve(2, lm, A, m.neq, F, perm, inv, kmax=30, lmax=200, tol=1e-12)
    r = F[:-1] - O.ebemv3_perm(lm, A, perm, inv, X)[:-1]
    assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(F[:-1])


def test_sink_stays_zero_and_sweeps_are_linear():
    m, A, F, lm, perm, inv = _problem(17)
    rng = np.random.default_rng(7)
    x = np.append(rng.standard_normal(m.neq), 0.0)
    y = np.append(rng.standard_normal(m.neq), 0.0)
    for kind in (1, 2, 3):
        a = O.elem_prec_apply(kind, lm, A, m.neq, x + 2.0 * y)
        b = O.elem_prec_apply(kind, lm, A, m.neq, x) + 2.0 * O.elem_prec_apply(kind, lm, A, m.neq, y)
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12)
