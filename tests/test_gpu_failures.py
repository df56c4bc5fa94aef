"""Failure handling without a GPU fault: bad numbers and exhausted limits come
back as status codes, and the library stays usable afterwards.

* a NaN in the right-hand side: the solve reports FG_ERR_BREAKDOWN (the
  reference's pgmres would divide by a NaN norm and carry on);
* a singular nodal block in the block-diagonal set-up
  (BlockDiag_precond_EBE_setup.c:90-147 inverts it by cofactors): the
  set-up returns FG_ERR_BREAKDOWN;
* a happy breakdown (the Krylov space holds the exact solution after one
  step: zero Hessenberg subdiagonal, pgmres.c:110-117) converges with the
  exact solution;
* a device-memory cap below what a system needs: creation fails with
  FG_ERR_NOMEM and succeeds once the cap is lifted.
(The bounded waits of the ILU kernels are covered in test_gpu_csr_ilu.py.)
"""
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


def test_nan_right_hand_side_is_breakdown(fg):
    p = G.transport_problem(17)
    A, F = O.build_k_f_supg(p)
    s = fg.System(p.mesh)
    s.set_blocks(A)
    Fp = s.precond_setup(fg.FG_PRECOND_DIAG, 0, F)
    Fp[5] = np.nan
    for prec in (fg.FG_PREC_FP64, fg.FG_PREC_MIXED):
        try:
            r = s.solve(Fp, tol=1e-10, precision=prec)
            assert r.stats["status"] == fg.FG_ERR_BREAKDOWN and r.stats["converged"] == 0
        except fg.FemGpuError as e:
            assert e.code == fg.FG_ERR_BREAKDOWN
    # the system still solves a good right-hand side
    Fp = s.precond_setup(fg.FG_PRECOND_DIAG, 0, F)
    r = s.solve(Fp, tol=1e-10, F_true=F)
    assert r.stats["converged"] == 1 and r.stats["status"] == 0


def test_singular_nodal_block_is_breakdown(fg):
    p = G.obliquo_problem(9)
    m = p.mesh
    A, R = O.build_euler(p)
    # zero every block entry of one interior node (a node with free dofs)
    node = next(i for i in range(m.nnodes) if all(m.type[4 * i + a] != 0 for a in range(4)))
    A = A.copy()
    for e in range(m.nel):
        for v in range(3):
            if m.ien[e][v] == node:
                blk = A[e].reshape(12, 12)
                blk[4 * v:4 * v + 4, :] = 0.0
                blk[:, 4 * v:4 * v + 4] = 0.0
    s = fg.System(m)
    s.set_blocks(A)
    with pytest.raises(fg.FemGpuError) as e:
        s.precond_setup(fg.FG_PRECOND_BLOCKDIAG, fg.FG_SETUP_REF_QUIRKS, R)
    assert e.value.code == fg.FG_ERR_BREAKDOWN
    # the unmodified blocks set up fine
    A0, R0 = O.build_euler(p)
    s.set_blocks(A0)
    s.precond_setup(fg.FG_PRECOND_BLOCKDIAG, fg.FG_SETUP_REF_QUIRKS, R0)


@pytest.mark.parametrize("precision", [64, 32])
def test_happy_breakdown_converges_exactly(fg, precision):
    """Diagonal element blocks with the Diag preconditioner: M^-1 A = I, so
    the first Arnoldi step finds h(2,1) = 0 and the solution is exact."""
    p = G.transport_problem(17)
    m = p.mesh
    A = np.zeros((m.nel, 9))
    A[:, [0, 4, 8]] = 1.0
    F = np.zeros(m.neq + 1)
    F[:-1] = np.random.default_rng(3).standard_normal(m.neq)
    s = fg.System(m)
    s.set_blocks(A)
    Fp = s.precond_setup(fg.FG_PRECOND_DIAG, 0, F.copy())
    r = s.solve(Fp, tol=1e-10, F_true=F, precision=precision)
    assert r.stats["converged"] == 1 and r.stats["status"] == 0
    assert r.stats["iterations"] <= (1 if precision == 64 else 4)
    d = s.diag()[:-1]
    assert np.allclose(r.x[:-1], F[:-1] / d, rtol=1e-12, atol=0)


def test_memory_limit_makes_creation_fail_cleanly(fg):
    p = G.transport_problem(65)
    used = fg.memory_in_use()
    try:
        fg.set_memory_limit(used + 4096)
        with pytest.raises(fg.FemGpuError) as e:
            fg.System(p.mesh)
        assert e.value.code == fg.FG_ERR_NOMEM
        assert fg.memory_in_use() == used          # nothing leaked by the failed creation
    finally:
        fg.set_memory_limit(0)
    s = fg.System(p.mesh)
    assert s.info()["n"] == p.mesh.neq
