"""The truncated SPIKE restatement (oracle/spike.c).  Its parity with the
reference is unpinned: the reference factorises each rank's block with
PARDISO, absent from the reference tree, and needs two or more MPI ranks.
It is pinned here by construction: with one block it is an exact banded LU
solve (checked against a sparse direct solve), with several blocks it is
exact on block-diagonal matrices, and it improves on Jacobi for the
transport operator."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G


def _csr(n=33, angle=40.0, k=1e-3):
    p = G.transport_problem(n, angle_deg=angle, k=k)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    perm, inv, _ = O.permutation_of_lm(m)
    IA, JA = O.csr_pattern(m, perm, inv)
    lm = O.fill_lm(m)
    lm_new = np.where(lm == m.neq, m.neq, inv[np.minimum(lm, m.neq)])
    AA = O.csr_assemble(lm_new, A, m.neq, IA, JA)
    M = sp.csr_matrix((AA[: len(JA)], JA, IA), shape=(m.neq, m.neq))
    return IA, JA, AA, M


def test_block_layout():
    IA, JA, AA, M = _csr()
    n = M.shape[0]
    s = O.Spike(IA, JA, AA, 8, 4)
    assert s.err == 0 and s.P == 4 and s.k == 8
    assert s.bs[0] == 0 and s.bs[-1] == n and np.all(np.diff(s.bs) >= 16)
    # bandwidths of the diagonal blocks from the matrix itself
    for q in range(s.P):
        b = M[s.bs[q]:s.bs[q + 1], s.bs[q]:s.bs[q + 1]].tocoo()
        d = b.row - b.col
        assert s.kl[q] == max(0, d.max()) and s.ku[q] == max(0, -d.min())
    # at most n / 2k blocks
    assert O.Spike(IA, JA, AA, 16, 10 ** 6).P == n // 32


def test_one_block_is_exact_lu():
    IA, JA, AA, M = _csr()
    f = np.random.default_rng(0).standard_normal(M.shape[0])
    z = O.Spike(IA, JA, AA, 8, 1).apply(f)
    e = spla.spsolve(M.tocsc(), f)
    assert np.linalg.norm(z - e) / np.linalg.norm(e) < 1e-12


def test_block_diagonal_matrix_is_exact():
    """No coupling between blocks: every block solve is exact."""
    IA, JA, AA, M = _csr(17)
    n = M.shape[0]
    P = 4
    bs = [n * q // P for q in range(P + 1)]
    blk = sp.block_diag([M[bs[q]:bs[q + 1], bs[q]:bs[q + 1]] for q in range(P)]).tocsr()
    blk.sort_indices()
    f = np.random.default_rng(1).standard_normal(n)
    z = O.Spike(blk.indptr.astype(np.int32), blk.indices.astype(np.int32), blk.data, 4, P).apply(f)
    e = spla.spsolve(blk.tocsc(), f)
    assert np.linalg.norm(z - e) / np.linalg.norm(e) < 1e-12


def test_corner_coupling_only_is_exact():
    """A matrix whose off-block entries all lie in the k x k corners and
    whose spikes vanish outside their tips: truncated SPIKE is exact when
    P = 2 (one interface, nothing truncated)."""
    IA, JA, AA, M = _csr(17)
    n = M.shape[0]
    bs = [0, n // 2, n]
    k = 6
    D = M.tolil()
    for i, j in zip(*M.nonzero()):
        qi, qj = int(i >= bs[1]), int(j >= bs[1])
        if qi != qj and not (abs(i - bs[1] + 0.5) < k and abs(j - bs[1] + 0.5) < k):
            D[i, j] = 0.0
    D = D.tocsr()
    D.eliminate_zeros()
    D.sort_indices()
    f = np.random.default_rng(3).standard_normal(n)
    z = O.Spike(D.indptr.astype(np.int32), D.indices.astype(np.int32), D.data, k, 2).apply(f)
    e = spla.spsolve(D.tocsc(), f)
    assert np.linalg.norm(z - e) / np.linalg.norm(e) < 1e-10


@pytest.mark.parametrize("P,k,factor", [(4, 8, 0.4), (8, 16, 0.4), (16, 4, 0.7)])
def test_better_than_jacobi(P, k, factor):
    IA, JA, AA, M = _csr()
    n = M.shape[0]
    f = np.random.default_rng(2).standard_normal(n)
    e = spla.spsolve(M.tocsc(), f)
    z = O.Spike(IA, JA, AA, k, P).apply(f)
    jac = f / M.diagonal()
    assert np.linalg.norm(z - e) < factor * np.linalg.norm(jac - e)


def test_rejects_bad_arguments():
    IA, JA, AA, M = _csr(9)
    with pytest.raises(ValueError):
        O.Spike(IA, JA, AA, 0, 4)
