"""The reference's entry points from libfemgpu_ns.so and libfemgpu_euler.so,
driven the way the NS Process loop (NS/Process.c:37-38) and Predictor_Old
(Predictor_Old.c:95-96) drive them: blocks filled by the driver's Build,
the block-diagonal set-up (F preconditioned in place), then pgmres with
mv = ebemvNDOF3/4 and the block-diagonal precond.  The set-up is bit-exact;
the solve follows the reference method (oracle) to rel-L2 1e-9 at tol 1e-10."""
import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G
import refapi

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _case(kind):
    if kind == "ns":
        p = G.cavity_problem(17, reynolds=100.0, jitter=0.2)
        u = np.random.default_rng(1).standard_normal(p.mesh.neq) * 0.1
        A, F = O.build_ns(p, u)
        return p.mesh, A, F, False
    p = G.obliquo_problem(17)
    u = p.initial_state() * (1 + 0.02 * np.random.default_rng(2).standard_normal(p.mesh.neq))
    A, F = O.build_euler(p, u)
    return p.mesh, A, F, True


@pytest.mark.parametrize("kind", ["ns", "euler"])
def test_block_drop_in_matches_reference_method(kind):
    m, A, F, quirks = _case(kind)
    st = refapi.BlockDriverState(kind, m, kmax=30, lmax=1000, tol=1e-10)
    st.Aaux[:] = A.reshape(-1)
    rc, Fp = st.precond_setup(F)
    assert rc == 0
    X0, it0, Fp0 = O.ebe_block_solve(m, A, F, 30, 1000, 1e-10, ref_quirks=quirks)
    assert np.array_equal(Fp[:-1], Fp0[:-1])
    rc, X = st.pgmres(Fp)
    assert rc == 0
    assert rel(X[:-1], X0[:-1]) <= 1e-9
    assert abs(st.P.iterations - it0) <= max(2, 0.02 * it0)
    Pv = np.random.default_rng(0).standard_normal(m.neq + 1)
    Pv[-1] = 0
    rc, Q = st.ebemv(Pv)
    assert rc == 0 and rel(Q[:-1], O.ebemv(O.fill_lm(m), A, m.neq, Pv)[:-1]) <= 1e-14
