"""The oracle's CSR path and ILU(0) against the reference's own
csr_Initialization, csr_assembly, csrmv and ILUp (bit-exact)."""
import os
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


ILUP = os.path.join(os.path.dirname(__file__), "golden", "ilup_sst.npz")


@pytest.mark.parametrize("key", ["n13_p1", "n13_p2", "n13_p3", "n17_p1", "n17_p2", "n17_p3"])
def test_ilup_bit_exact(key, oracle_lib):
    """ILU(p) (level-of-fill symbolic pass, numeric factorisation and the
    substitutions) against the reference's "ILU<p>" applied to a vector."""
    d = np.load(ILUP)
    p = int(key.split("_p")[1])
    FIA, FJA, FDG, LU, D = O.ilup(d[key + "_IA"], d[key + "_JA"], d[key + "_AA"], p)
    x = O.ilup_apply(FIA, FJA, FDG, LU, D, d[key + "_P"])
    assert np.array_equal(x, d[key + "_z"])
    assert FIA[-1] > len(d[key + "_JA"])          # fill entered


def test_ilup_level0_is_ilu0(oracle_lib):
    d = np.load(ILUP)
    IA, JA, AA = d["n13_p1_IA"], d["n13_p1_JA"], d["n13_p1_AA"]
    FIA, FJA, FDG, LU, D = O.ilup(IA, JA, AA, 0)
    rc, LU0, D0 = O.ilu0(IA, JA, AA)
    y = d["n13_p1_P"]
    assert np.array_equal(FIA, IA) and np.array_equal(FJA, JA)
    assert np.array_equal(O.ilup_apply(FIA, FJA, FDG, LU, D, y), O.ilu0_apply(IA, JA, LU0, D0, y)[: len(IA) - 1])
