"""The reference's entry points from libfemgpu_sst.so, driven the way the
steady-transport Process loop drives them (Process.c:59-76): blocks filled
by the driver, Diag_precond_EBE_setup, then pgmres with mv = ebemv and
precond = Diag_precond.  Results follow the reference method (oracle):
rel-L2 <= 1e-9 at tol 1e-10, Diag accumulating across set-ups."""
import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G
import refapi

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_drop_in_pgmres_matches_reference_method():
    p = G.transport_problem(33)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    st = refapi.DriverState(m)
    st.Aaux[:] = A.reshape(-1)                       # what Build_K_F_SUPG leaves in Aaux
    rc, Fp = st.precond_setup(F)
    assert rc == 0
    D0, inv0, Fp0 = O.diag_setup(lm, A, m.neq, F)
    assert np.array_equal(st.Diag[:-1], D0[:-1])
    assert np.array_equal(Fp[:-1], Fp0[:-1])
    rc, X = st.pgmres(Fp)
    assert rc == 0
    X0, it0, *_ = O.ebe_diag_solve(lm, A, m.neq, F, perm, inv, kmax=30, lmax=1000, tol=1e-10)
    assert rel(X[:-1], X0[:-1]) <= 1e-9
    assert abs(st.P.iterations - it0) <= 2
    # ebemv through the shim
    Pv = np.random.default_rng(0).standard_normal(m.neq + 1)
    Pv[-1] = 0
    rc, Q = st.ebemv(Pv)
    assert rc == 0 and rel(Q[:-1], O.ebemv3_perm(lm, A, perm, inv, Pv)[:-1]) <= 1e-14
    # a second set-up accumulates Diag, as the reference's never-cleared Diag
    rc, Fp2 = st.precond_setup(F)
    D1, _, Fp1 = O.diag_setup(lm, A, m.neq, F, Diag=D0.copy())
    assert np.array_equal(st.Diag[:-1], D1[:-1]) and np.array_equal(Fp2[:-1], Fp1[:-1])


@pytest.mark.parametrize("precond", ["ILU0", "SPIKE8"])
def test_drop_in_csr_storage(precond):
    """MatrixVectorProductScheme "CSR": the driver's csr_assembly calls,
    ILUp_precond_setup / SPIKE_precond_setup and pgmres with mv = csrmv, all
    from the shim.  The preconditioned F is bit-exact against the oracle's
    ILU(0) / SPIKE on the reference's CSR matrix; GMRES reaches the
    reference method's solution."""
    p = G.transport_problem(33)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    IA, JA = O.csr_pattern(m, perm, inv)
    lm_new = np.where(lm == m.neq, m.neq, inv[np.minimum(lm, m.neq)])
    AA = O.csr_assemble(lm_new, A, m.neq, IA, JA)
    st = refapi.DriverState(m, precond=precond, scheme="CSR")
    st.csr_assembly(A)                               # what Build_K_F_SUPG does with CSR storage
    rc, Fp = st.precond_setup(F)
    assert rc == 0
    Fi = F[:-1][perm[:-1]]
    if precond == "ILU0":
        rc0, LU, D = O.ilu0(IA, JA, AA)
        zi = O.ilu0_apply(IA, JA, LU, D, np.append(Fi, 0.0))[:-1]
    else:
        zi = O.Spike(IA, JA, AA, 8, 16).apply(Fi)
        assert st.P.k_SPIKE_block_size == 8
    assert np.array_equal(Fp[:-1][perm[:-1]], zi)
    rc, X = st.pgmres(Fp)
    assert rc == 0
    X0, it0, *_ = O.ebe_diag_solve(lm, A, m.neq, F, perm, inv, kmax=30, lmax=1000, tol=1e-12)
    assert rel(X[:-1], X0[:-1]) <= 1e-8
    Pv = np.random.default_rng(1).standard_normal(m.neq + 1)
    Pv[-1] = 0
    rc, Q = st.csrmv(Pv)
    assert rc == 0 and rel(Q[:-1], O.ebemv3_perm(lm, A, perm, inv, Pv)[:-1]) <= 1e-14
