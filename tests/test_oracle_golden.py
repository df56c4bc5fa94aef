"""The oracle (CPU restatement) against the golden fixtures generated from
the reference's own C, and against the reference build itself where it is
present.  Integer and index work and the element/right-hand-side arithmetic
are bit-exact; so is the whole Process loop (same rounding, same order)."""
import glob
import os

import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "sst_*.npz")))


def _problem(g):
    m = G.Mesh(g["x"], g["y"], g["ien"], 1, g["type"], g["invp"], int(g["neq"]))
    return G.TransportProblem(m, float(g["k"]), float(g["gamma"]), tuple(g["beta"]), float(g["f"]),
                              g["upresc"], int(g["upmode"]), float(g["upval"]), True)


@pytest.fixture(scope="module", params=GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def case(request, oracle_lib):
    g = dict(np.load(request.param))
    return g, _problem(g)


def test_golden_present():
    assert len(GOLDEN) >= 3


def test_connectivity_bit_exact(case):
    g, p = case
    assert np.array_equal(O.fill_lm(p.mesh), g["lm"])
    perm, inv, band = O.permutation_of_lm(p.mesh)
    assert np.array_equal(perm, g["perm"]) and np.array_equal(inv, g["invperm"])
    assert np.array_equal(band, g["band"])


def test_assembly_bit_exact(case):
    g, p = case
    A, F = O.build_k_f_supg(p)
    assert np.array_equal(A, g["A"])
    assert np.array_equal(F[: p.mesh.neq], g["F"])


def test_diag_gmres_bit_exact(case):
    g, p = case
    X, it, Diag, invDiag, Fp = O.ebe_diag_solve(g["lm"], g["A"], p.mesh.neq, np.append(g["F"], 0.0),
                                                g["perm"], g["invperm"], kmax=30, lmax=1000, tol=1e-10)
    assert it == int(g["gmres_its"])
    assert np.array_equal(Fp[: p.mesh.neq], g["Fp"])
    assert np.array_equal(X[: p.mesh.neq], g["X"])


def test_process_bit_exact(case):
    g, p = case
    U, nl, its = O.transport_process(p, 1e-10, 1e-3, 30, 1000)
    assert its == int(g["process_its"])
    assert np.array_equal(U, g["U"])


def test_teste_known_answer():
    """TESTE (01_SS_Transport_Equation/2D/TESTE): k = 1, beta = 0, f = 0,
    u = 10 on the boundary: the exact solution is u = 10."""
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "sst_9_teste.npz")))
    assert np.max(np.abs(g["U"] - 10.0)) < 1e-8


@pytest.mark.skipif(not O.ref_available(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("n,angle,k", [(5, 30.0, 1e-6), (33, 123.0, 1e-4), (65, 250.0, 1e-8)])
def test_oracle_vs_reference_build(n, angle, k):
    p = G.transport_problem(n, angle_deg=angle, k=k)
    m = p.mesh
    lm_r, perm_r, inv_r, band_r, nnz = O.ref_connectivity(m)
    perm, inv, band = O.permutation_of_lm(m)
    assert np.array_equal(O.fill_lm(m), lm_r)
    assert np.array_equal(perm, perm_r) and np.array_equal(inv, inv_r) and np.array_equal(band, band_r)
    u = np.random.default_rng(n).random(m.neq)
    A, F = O.build_k_f_supg(p, u)
    A_r, F_r = O.ref_build(p, u)
    assert np.array_equal(A, A_r) and np.array_equal(F[: m.neq], F_r[: m.neq])
    P = np.random.default_rng(1).random(m.neq + 1)
    P[-1] = 0
    assert np.array_equal(O.ebemv3_perm(lm_r, A, perm, inv, P)[: m.neq], O.ref_ebemv(lm_r, A, perm_r, inv_r, P)[: m.neq])
    if n <= 33:
        U, nl, its = O.transport_process(p, 1e-10, 1e-3, 30, 1000)
        U_r, its_r = O.ref_process(p, 1e-10, 1e-3, 30, 1000)
        assert its == its_r and np.array_equal(U, U_r)


@pytest.mark.skipif(not O.ref_available(), reason="reference build (oracle/_ref) not present")
def test_symrcm_vs_reference_on_irregular_graphs():
    """RCM tie-breaking on patterns other than the structured mesh: a jittered
    mesh's adjacency with random symmetric extra couplings and two components."""
    rng = np.random.default_rng(5)
    for trial in range(5):
        n = int(rng.integers(20, 200))
        A = np.zeros((n, n), dtype=bool)
        A[np.arange(n), np.arange(n)] = True
        for _ in range(3 * n):
            i, j = rng.integers(0, n // 2 if trial % 2 else n, size=2)
            A[i, j] = A[j, i] = True
        IA = np.concatenate([[0], np.cumsum(A.sum(1))]).astype(np.int32)
        JA = np.concatenate([np.nonzero(r)[0] for r in A]).astype(np.int32)
        assert np.array_equal(O.symrcm(IA, JA), O.ref_symrcm(IA, JA))


def test_structured_mesh_matches_generator_order(oracle_lib):
    """Python mesh = oracle's restatement of meshGenerator.c's node/triangle order."""
    import ctypes
    for M, left in ((4, 0), (7, 1)):
        x = np.empty((M + 1) ** 2)
        y = np.empty((M + 1) ** 2)
        ien = np.empty(2 * M * M * 3, dtype=np.int32)
        O.lib().or_mesh_structured(M, M, 0.0, 0.0, 1.0, 1.0, left, x, y, ien)
        X, Y, I = G.structured_mesh(M, M, left=bool(left))
        assert np.array_equal(X, x) and np.array_equal(Y, y) and np.array_equal(I.reshape(-1), ien)


DD = os.path.join(os.path.dirname(__file__), "golden", "dd_sst.npz")


@pytest.mark.parametrize("name", ["sst_17_adv", "sst_12_mixed"])
@pytest.mark.parametrize("shock", [1, 2], ids=["cau", "caudd"])
def test_dd_bit_exact(name, shock, oracle_lib):
    """StabilizationForm "DD" (Build_K_F_DD with CAU or CAUDD): blocks, F and
    the whole Process loop against the reference's own run."""
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz")))
    p = _problem(g)
    p.form, p.cau = 1, shock
    d = np.load(DD)
    key = f"{name}_c{shock}"
    A, F = O.build_k_f_supg(p, d[key + "_u"])
    assert np.array_equal(A, d[key + "_A"])
    assert np.array_equal(F[: p.mesh.neq], d[key + "_F"])
    U, nl, its = O.transport_process(p, 1e-10, 1e-3, 30, 1000)
    assert its == int(d[key + "_its"])
    assert np.array_equal(U, d[key + "_U"])


def test_dd_against_reference_build(oracle_lib):
    if not O.ref_available():
        pytest.skip("reference build (oracle/_ref) not present")
    p = G.transport_problem(21, angle_deg=110.0, k=1e-4, gamma=0.2, f=0.5, cau=2)
    p.form = 1
    u = np.random.default_rng(21).random(p.mesh.neq)
    A0, F0 = O.ref_build(p, u)
    A1, F1 = O.build_k_f_supg(p, u)
    assert np.array_equal(A0, A1) and np.array_equal(F0[:-1], F1[:-1])


SHOCK = os.path.join(os.path.dirname(__file__), "golden", "shock_sst.npz")
SHOCK_CASES = [(0, 3, 0), (0, 3, 1), (0, 1, 2), (1, 3, 2), (1, 2, 1), (1, 3, 0)]   # (form, shock, h_shock)


@pytest.mark.parametrize("form,shock,hs", SHOCK_CASES)
def test_shock_options_bit_exact(form, shock, hs, oracle_lib):
    """ShockCapture "YZBeta" (with its per-element state across the Process
    loop) and h_Shock "Option1" / "Option2", both forms, against the
    reference's own runs."""
    p = G.transport_problem(13, angle_deg=110.0, k=1e-4, gamma=0.2, f=0.5, cau=shock)
    p.form, p.h_shock = form, hs
    d = np.load(SHOCK)
    key = f"f{form}_c{shock}_h{hs}"
    A, F = O.build_k_f_supg(p, d[key + "_u"])
    assert np.array_equal(A, d[key + "_A"]) and np.array_equal(F[: p.mesh.neq], d[key + "_F"])
    U, nl, its = O.transport_process(p, 1e-10, 1e-3, 30, 1000)
    assert its == int(d[key + "_its"]) and np.array_equal(U, d[key + "_U"])
