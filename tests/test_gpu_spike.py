"""Truncated SPIKE on the GPU (FG_PRECOND_SPIKE) against its CPU
restatement (oracle/spike.c): the set-up applied to F and the FP64 apply
are bit-exact (same operation order, no FMA contraction on either side);
GMRES with SPIKE reaches the Diag solution at tol 1e-10 in fewer
iterations, in FP64 and mixed precision; a system solved inside a batch is
bit-identical to the same solve alone."""
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


def _setup(fg, n, k, parts, angle=40.0, kappa=1e-3):
    p = G.transport_problem(n, angle_deg=angle, k=kappa)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    perm, inv, _ = O.permutation_of_lm(m)
    s = fg.System(m)
    s.set_blocks(A)
    s.set_operator(fg.FG_OP_CSR)
    s.set_spike(k, parts)
    IA, JA, AA = s.csr()
    return p, m, A, F, perm, inv, s, O.Spike(IA, JA, AA, k, parts)


@pytest.mark.parametrize("n,k,parts", [(17, 4, 1), (33, 8, 4), (66, 16, 8), (66, 4, 16), (90, 64, 3)])
def test_spike_setup_and_apply_bit_exact(fg, n, k, parts):
    p, m, A, F, perm, inv, s, ref = _setup(fg, n, k, parts)
    assert ref.err == 0
    Fp = s.precond_setup(fg.FG_PRECOND_SPIKE, 0, F)
    zi = ref.apply(F[:-1][perm[:-1]])            # oracle in the internal (CSR) numbering
    assert np.array_equal(Fp[:-1][perm[:-1]], zi)
    v = np.random.default_rng(n).standard_normal(m.neq + 1)
    v[-1] = 0
    z = s.precond_apply(v)
    assert np.array_equal(z[:-1][perm[:-1]], ref.apply(v[:-1][perm[:-1]]))


def test_spike_large_blocks_in_global_memory(fg):
    """Blocks above 6144 rows keep their working vector in global memory."""
    p, m, A, F, perm, inv, s, ref = _setup(fg, 130, 8, 2)
    assert np.diff(ref.bs).max() > 6144
    v = np.random.default_rng(5).standard_normal(m.neq + 1)
    v[-1] = 0
    s.precond_setup(fg.FG_PRECOND_SPIKE, 0, None)
    z = s.precond_apply(v)
    assert np.array_equal(z[:-1][perm[:-1]], ref.apply(v[:-1][perm[:-1]]))


def test_spike_wide_band(fg):
    """Bandwidth above the 256 threads of an apply CTA (rows beyond them take
    the plain loop) and 64 blocks."""
    p, m, A, F, perm, inv, s, ref = _setup(fg, 264, 8, 64)
    assert ref.kl.max() > 256 and ref.P == 64
    Fp = s.precond_setup(fg.FG_PRECOND_SPIKE, 0, F)
    assert np.array_equal(Fp[:-1][perm[:-1]], ref.apply(F[:-1][perm[:-1]]))


@pytest.mark.parametrize("precision", [64, 32])
def test_gmres_spike(fg, precision):
    p, m, A, F, perm, inv, s, ref = _setup(fg, 65, 16, 8, angle=30.0, kappa=1e-6)
    lm = O.fill_lm(m)
    X0, it0, *_ = O.ebe_diag_solve(lm, A, m.neq, F, perm, inv, kmax=30, lmax=1000, tol=1e-12)
    Fp = s.precond_setup(fg.FG_PRECOND_SPIKE, 0, F)
    r = s.solve(Fp, tol=1e-10, F_true=F, precision=precision)
    assert r.stats["converged"] == 1 and r.stats["status"] == 0
    assert r.stats["iterations"] < it0           # SPIKE needs fewer steps than Diag
    res = np.linalg.norm(F[:-1] - O.ebemv3_perm(lm, A, perm, inv, r.x)[:-1]) / np.linalg.norm(F[:-1])
    if precision == 32:
        assert res <= 1e-10
    assert np.linalg.norm(r.x[:-1] - X0[:-1]) / np.linalg.norm(X0[:-1]) <= 1e-8


@pytest.mark.parametrize("precision", [64, 32])
def test_spike_batch_equals_alone(fg, precision):
    cases = [_setup(fg, n, 8, parts, angle=a) for n, parts, a in ((33, 4, 10.0), (40, 1, 200.0), (50, 6, 95.0))]
    systems, Bs, Fs = [], [], []
    for p, m, A, F, perm, inv, s, ref in cases:
        Bs.append(s.precond_setup(fg.FG_PRECOND_SPIKE, 0, F))
        Fs.append(F)
        systems.append(s)
    Xb, stb = fg.solve_batch(systems, Bs, Fs, precision=precision)
    for s, B, F, X, st in zip(systems, Bs, Fs, Xb, stb):
        r = s.solve(B, F_true=F, precision=precision)
        assert st["converged"] == 1
        assert st["iterations"] == r.stats["iterations"]
        assert np.array_equal(X, r.x)


def test_spike_needs_csr_and_valid_sizes(fg):
    p = G.transport_problem(17)
    A, F = O.build_k_f_supg(p)
    s = fg.System(p.mesh)
    s.set_blocks(A)
    with pytest.raises(fg.FemGpuError):
        s.precond_setup(fg.FG_PRECOND_SPIKE, 0, F)
    with pytest.raises(fg.FemGpuError):
        s.set_spike(0, 4)
    with pytest.raises(fg.FemGpuError):
        s.set_spike(65, 4)
