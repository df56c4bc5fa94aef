"""The oracle's CSR path and ILU(0) against the reference's own
csr_Initialization, csr_assembly, csrmv and ILUp (bit-exact)."""
import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G


@pytest.mark.skipif(not O.ref_available(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("n,angle,k", [(9, 40.0, 1e-3), (33, 200.0, 1e-6), (48, 300.0, 1e-2)])
def test_csr_and_ilu0_match_reference(n, angle, k):
    p = G.transport_problem(n, angle_deg=angle, k=k)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    perm, inv, _ = O.permutation_of_lm(m)
    P = np.random.default_rng(n).standard_normal(m.neq + 1)
    P[-1] = 0
    IA_r, JA_r, AA_r, invp_r, Q_r, z_r = O.ref_csr(p, A, P)
    IA, JA = O.csr_pattern(m, perm, inv)
    lm = O.fill_lm(m)
    lm_new = np.where(lm == m.neq, m.neq, inv[np.minimum(lm, m.neq)])
    AA = O.csr_assemble(lm_new, A, m.neq, IA, JA)
    assert np.array_equal(IA, IA_r) and np.array_equal(JA, JA_r) and np.array_equal(AA, AA_r)
    free = m.type != 0
    assert np.array_equal(inv[m.invp[free]], invp_r[free])      # csr_Initialization renumbering
    assert np.array_equal(O.csrmv(IA, JA, AA, P)[:-1], Q_r[:-1])
    rc, LU, D = O.ilu0(IA, JA, AA)
    assert rc == 0
    assert np.array_equal(O.ilu0_apply(IA, JA, LU, D, P)[:-1], z_r[:-1])
