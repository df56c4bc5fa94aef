"""Assembled CSR operator and ILU(0) on the GPU against the oracle, which
is pinned bit-exactly to the reference's csr_Initialization, csr_assembly,
csrmv and ILUp (tests/test_oracle_csr.py).  CSR pattern, values and the
ILU(0) set-up (factorisation applied to F, FP64, no FMA contraction) are
bit-exact; the SpMV sums a row in lane order (relative 1e-14 in FP64,
1e-5 in FP32); GMRES with ILU(0) reaches the reference method's solution
to rel-L2 1e-9 at tol 1e-10."""
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


def _setup(fg, n, angle=40.0, k=1e-3):
    p = G.transport_problem(n, angle_deg=angle, k=k)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    perm, inv, _ = O.permutation_of_lm(m)
    IA, JA = O.csr_pattern(m, perm, inv)
    lm = O.fill_lm(m)
    lm_new = np.where(lm == m.neq, m.neq, inv[np.minimum(lm, m.neq)])
    AA = O.csr_assemble(lm_new, A, m.neq, IA, JA)
    s = fg.System(m)
    s.set_blocks(A)
    s.set_operator(fg.FG_OP_CSR)
    return p, m, A, F, perm, inv, IA, JA, AA, lm, s


@pytest.mark.parametrize("n", [9, 33, 66])
def test_csr_structure_and_values_bit_exact(fg, n):
    p, m, A, F, perm, inv, IA, JA, AA, lm, s = _setup(fg, n)
    IAg, JAg, AAg = s.csr()
    assert np.array_equal(IAg, IA) and np.array_equal(JAg, JA) and np.array_equal(AAg, AA)


@pytest.mark.parametrize("n", [17, 66])
def test_csr_matvec(fg, n):
    p, m, A, F, perm, inv, IA, JA, AA, lm, s = _setup(fg, n)
    P = np.random.default_rng(n).standard_normal(m.neq + 1)
    P[-1] = 0
    ref = O.ebemv3_perm(lm, A, perm, inv, P)          # reference numbering
    assert rel(s.matvec(P)[:-1], ref[:-1]) < 1e-14
    assert rel(s.matvec(P, 32)[:-1], ref[:-1]) < 1e-5


@pytest.mark.parametrize("ndof", [3, 4])
def test_csr_matvec_multidof(fg, ndof):
    m = G.multi_dof_mesh(9, ndof, seed=ndof)
    A = G.random_blocks(m.nel, 3 * ndof, seed=ndof)
    s = fg.System(m)
    s.set_blocks(A)
    s.set_operator(fg.FG_OP_CSR)
    P = np.random.default_rng(2).standard_normal(m.neq + 1)
    P[-1] = 0
    assert rel(s.matvec(P)[:-1], O.ebemv(O.fill_lm(m), A, m.neq, P)[:-1]) < 1e-14


@pytest.mark.parametrize("n", [17, 66])
def test_ilu0_setup_bit_exact(fg, n):
    p, m, A, F, perm, inv, IA, JA, AA, lm, s = _setup(fg, n)
    rc, LU, D = O.ilu0(IA, JA, AA)
    assert rc == 0
    Fp = s.precond_setup(fg.FG_PRECOND_ILU0, 0, F)
    # the oracle works in the CSR (internal) numbering: map F there and back
    Fi = np.append(F[:-1][perm[:-1]], 0.0)
    zi = O.ilu0_apply(IA, JA, LU, D, Fi)
    z = np.zeros(m.neq + 1)
    z[perm[:-1]] = zi[:-1]
    assert np.array_equal(Fp[:-1], z[:-1])
    q = s.precond_apply(F)
    assert rel(q[:-1], z[:-1]) < 1e-14


@pytest.mark.parametrize("precision", [64, 32])
def test_gmres_ilu0(fg, precision):
    p, m, A, F, perm, inv, IA, JA, AA, lm, s = _setup(fg, 65, angle=30.0, k=1e-6)
    X0, it0, *_ = O.ebe_diag_solve(lm, A, m.neq, F, perm, inv, kmax=30, lmax=1000, tol=1e-12)
    Fp = s.precond_setup(fg.FG_PRECOND_ILU0, 0, F)
    r = s.solve(Fp, tol=1e-10, F_true=F, precision=precision)
    assert r.stats["converged"] == 1 and r.stats["status"] == 0
    assert r.stats["iterations"] < it0          # ILU(0) needs fewer steps than Diag
    res = np.linalg.norm(F[:-1] - O.ebemv3_perm(lm, A, perm, inv, r.x)[:-1]) / np.linalg.norm(F[:-1])
    if precision == 32:
        assert res <= 1e-10
    assert rel(r.x[:-1], X0[:-1]) <= 1e-8


@pytest.mark.parametrize("lev", [1, 2])
def test_ilup_setup_bit_exact(fg, lev):
    """ILU(p) (Preconditioner "ILU<p>"): the device factor pattern,
    factorisation and substitutions against the oracle (pinned to the
    reference's ILUp)."""
    p, m, A, F, perm, inv, IA, JA, AA, lm, s = _setup(fg, 33)
    FIA, FJA, FDG, LU, D = O.ilup(IA, JA, AA, lev)
    s.set_ilu_fill(lev)
    Fp = s.precond_setup(fg.FG_PRECOND_ILU0, 0, F)
    Fi = np.append(F[:-1][perm[:-1]], 0.0)
    zi = O.ilup_apply(FIA, FJA, FDG, LU, D, Fi)
    z = np.zeros(m.neq + 1)
    z[perm[:-1]] = zi
    assert np.array_equal(Fp[:-1], z[:-1])


def test_gmres_ilup_fewer_iterations(fg):
    p, m, A, F, perm, inv, IA, JA, AA, lm, s = _setup(fg, 65, angle=30.0, k=1e-6)
    its = []
    for lev in (0, 2):
        s.set_ilu_fill(lev)
        Fp = s.precond_setup(fg.FG_PRECOND_ILU0, 0, F)
        r = s.solve(Fp, tol=1e-10, F_true=F, precision=64)
        assert r.stats["converged"] == 1
        res = np.linalg.norm(F[:-1] - O.ebemv3_perm(lm, A, perm, inv, r.x)[:-1]) / np.linalg.norm(F[:-1])
        assert res <= 1e-9
        its.append(r.stats["iterations"])
    assert its[1] <= its[0]


@pytest.mark.parametrize("blocks,lev", [(1, 0), (4, 0), (16, 0), (8, 1)])
def test_block_jacobi_ilu_bit_exact(fg, blocks, lev):
    """Block-Jacobi ILU(p) over equal row blocks of the RCM-ordered CSR
    operator (each block factorised by itself, as each MPI rank of the
    reference does) against the oracle's ILU(p) of the block-diagonal
    matrix; one block is the global ILU(p)."""
    p, m, A, F, perm, inv, IA, JA, AA, lm, s = _setup(fg, 33)
    BIA, BJA, BAA = O.block_diagonal_csr(IA, JA, AA, blocks)
    FIA, FJA, FDG, LU, D = O.ilup(BIA, BJA, BAA, lev)
    s.set_ilu_fill(lev)
    s.set_ilu_blocks(blocks)
    Fp = s.precond_setup(fg.FG_PRECOND_ILU0, 0, F)
    Fi = np.append(F[:-1][perm[:-1]], 0.0)
    zi = O.ilup_apply(FIA, FJA, FDG, LU, D, Fi)
    z = np.zeros(m.neq + 1)
    z[perm[:-1]] = zi[:m.neq]
    assert np.array_equal(Fp[:-1], z[:-1])


def test_block_jacobi_ilu_gmres(fg):
    """GMRES with block-Jacobi ILU(0): converges to the FP64 solution, with
    more iterations than the global ILU(0) and fewer than Diag."""
    p, m, A, F, perm, inv, IA, JA, AA, lm, s = _setup(fg, 65, angle=30.0, k=1e-6)
    X0, it0, *_ = O.ebe_diag_solve(lm, A, m.neq, F, perm, inv, kmax=30, lmax=1000, tol=1e-12)
    its = []
    for blocks in (1, 16):
        s.set_ilu_blocks(blocks)
        Fp = s.precond_setup(fg.FG_PRECOND_ILU0, 0, F)
        r = s.solve(Fp, tol=1e-10, F_true=F, precision=64)
        assert r.stats["converged"] == 1
        assert rel(r.x[:-1], X0[:-1]) <= 1e-8
        its.append(r.stats["iterations"])
    assert its[0] <= its[1] < it0


def test_ilu_wait_limit_times_out_and_recovers(fg):
    """A one-poll limit on the ILU kernels' dependency waits: the set-up
    returns FG_ERR_TIMEOUT instead of waiting (the waits end; nothing
    hangs), and with the default limit back the same set-up succeeds."""
    p, m, A, F, perm, inv, IA, JA, AA, lm, s = _setup(fg, 129)
    try:
        fg.set_wait_limit(1)
        with pytest.raises(fg.FemGpuError) as e:
            s.precond_setup(fg.FG_PRECOND_ILU0, 0, F)
        assert e.value.code == fg.FG_ERR_TIMEOUT
    finally:
        fg.set_wait_limit()
    Fp = s.precond_setup(fg.FG_PRECOND_ILU0, 0, F)
    assert np.all(np.isfinite(Fp))
