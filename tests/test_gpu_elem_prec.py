"""The element preconditioners "LUe" and "SGSe" on the GPU against the
oracle (itself bit-identical with the reference's LU_precond_EBE*.c and
SGS_precond_EBE*.c, tests/test_oracle_elem_prec.py).

* set-up: the preconditioned right-hand side M^-1 F, bit for bit;
* one application of the left sweep (LU, SGS forward) and of the right
  sweep (SGS backward; the identity for LUe), bit for bit;
* pgmres with the left / right pair (pgmres.c:61,93,186: precondR before
  every matvec and on X at the end): iterations within +-2 of the
  oracle's modified Gram-Schmidt and the solution to 1e-9, with the true
  residual of A x = F;
* a batch equals its members solved alone, bit for bit; the mixed
  precision solver refuses the sequential sweeps (FG_ERR_UNSUPPORTED).
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


def _setup(fg, n, angle=30.0, k=1e-3):
    p = G.transport_problem(n, angle_deg=angle, k=k)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    s = fg.System(m)
    s.set_blocks(A)
    return p, m, A, F, lm, perm, inv, s


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("n", [17, 33])
@pytest.mark.parametrize("kind", ["lue", "sgse"])
def test_setup_and_sweeps_bit_exact(fg, n, kind):
    p, m, A, F, lm, perm, inv, s = _setup(fg, n)
    pk = fg.FG_PRECOND_LUE if kind == "lue" else fg.FG_PRECOND_SGSE
    left = 1 if kind == "lue" else 2
    Fp = s.precond_setup(pk, 0, F)
    assert np.array_equal(Fp[:-1], O.elem_prec_apply(left, lm, A, m.neq, F)[:-1])
    z = np.append(np.random.default_rng(n).standard_normal(m.neq), 0.0)
    assert np.array_equal(s.precond_apply(z)[:-1], O.elem_prec_apply(left, lm, A, m.neq, z)[:-1])
    zr = s.precond_apply_right(z)
    want = z if kind == "lue" else O.elem_prec_apply(3, lm, A, m.neq, z)
    assert np.array_equal(zr[:-1], want[:-1])


@pytest.mark.parametrize("kind", ["lue", "sgse"])
def test_gmres_matches_oracle(fg, kind):
    p, m, A, F, lm, perm, inv, s = _setup(fg, 33)
    pk, ok = (fg.FG_PRECOND_LUE, 1) if kind == "lue" else (fg.FG_PRECOND_SGSE, 2)
    X0, it0, Fp0 = O.ebe_elem_solve(ok, lm, A, m.neq, F, perm, inv, kmax=30, lmax=200, tol=1e-10)
    Fp = s.precond_setup(pk, 0, F)
    assert np.array_equal(Fp[:-1], Fp0[:-1])
    r = s.solve(Fp, kmax=30, lmax=200, tol=1e-10, F_true=F)
    assert r.stats["converged"] == 1 and r.stats["status"] == 0
    assert abs(r.stats["iterations"] - it0) <= 2
    assert rel(r.x[:-1], X0[:-1]) <= 1e-9
    res = np.linalg.norm(F[:-1] - O.ebemv3_perm(lm, A, perm, inv, r.x)[:-1]) / np.linalg.norm(F[:-1])
    assert res <= 1e-8
    assert abs(r.stats["true_rel_residual"] - res) <= 1e-12 + 1e-6 * res


def test_batch_equals_alone_and_mixed_refused(fg):
    sys_, Fs, xs = [], [], []
    for n, ang in ((17, 20.0), (25, 60.0)):
        p, m, A, F, lm, perm, inv, s = _setup(fg, n, angle=ang)
        Fp = s.precond_setup(fg.FG_PRECOND_SGSE, 0, F)
        xs.append(s.solve(Fp, kmax=30, lmax=200, tol=1e-10).x)
        sys_.append(s)
        Fs.append(Fp)
    Xb, stb = fg.solve_batch(sys_, Fs, kmax=30, lmax=200, tol=1e-10, precision=fg.FG_PREC_FP64)
    for x, xb in zip(xs, Xb):
        assert np.array_equal(x, xb)
    with pytest.raises(fg.FemGpuError) as e:
        sys_[0].solve(Fs[0], kmax=30, lmax=200, tol=1e-10, precision=fg.FG_PREC_MIXED)
    assert e.value.code == fg.FG_ERR_UNSUPPORTED
