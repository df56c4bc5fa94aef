"""Batched solves: every member's result is bit-identical to solving it
alone (the reductions of a system depend only on its own parts), for both
precisions, through the host-buffer and the device-resident entry points."""
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


def _problems():
    return [G.transport_problem(n, angle_deg=a, k=k) for n, a, k in
            [(17, 30.0, 1e-6), (33, 200.0, 1e-3), (9, 95.0, 1e-8), (65, 315.0, 1e-5), (40, 10.0, 1e-2)]]


@pytest.mark.parametrize("precision", [64, 32])
def test_batch_equals_alone(fg, precision):
    probs = _problems()
    systems, Bs, Fs = [], [], []
    for p in probs:
        A, F = O.build_k_f_supg(p)
        s = fg.System(p.mesh)
        s.set_blocks(A)
        Bs.append(s.precond_setup(fg.FG_PRECOND_DIAG, 0, F))
        Fs.append(F)
        systems.append(s)
    Xb, stb = fg.solve_batch(systems, Bs, Fs, precision=precision)
    for s, B, F, X, st in zip(systems, Bs, Fs, Xb, stb):
        r = s.solve(B, F_true=F, precision=precision)
        assert st["converged"] == 1
        assert st["iterations"] == r.stats["iterations"]
        assert np.array_equal(X, r.x)


def test_resident_equals_host_path(fg):
    probs = _problems()[:3]
    systems = [fg.transport_system(p) for p in probs]
    for s, p in zip(systems, probs):
        s.transport_prepare(p)
    st = fg.solve_resident(systems, precision=32)
    for s, p, r in zip(systems, probs, st):
        F = s.transport_assemble(p)
        B = s.precond_setup(fg.FG_PRECOND_DIAG, 0, F)
        ref = s.solve(B, F_true=F, precision=32)
        assert r["iterations"] == ref.stats["iterations"]
        assert np.array_equal(s.solution(), ref.x)


def test_launch_count_grows(fg):
    p = G.transport_problem(9)
    s = fg.transport_system(p)
    before = fg.launch_count()
    s.transport_prepare(p)
    fg.solve_resident([s])
    assert fg.launch_count() > before


def test_mixed16_basis_converges(fg):
    """FP16 storage of the Krylov basis (FP32 arithmetic, FP64 refinement):
    the batch reaches the same true relative residual and the FP64 solution."""
    probs = G.batch_transport_problems(count=6, seed=7, nmin=17, nmax=97)
    systems, Bs, Fs = [], [], []
    for p in probs:
        s = fg.transport_system(p)
        F = s.transport_assemble(p)
        Fp = s.precond_setup(fg.FG_PRECOND_DIAG, fg.FG_SETUP_ACCUMULATE, F)
        systems.append(s); Bs.append(Fp); Fs.append(F)
    X64, st64 = fg.solve_batch(systems, Bs, Fs, kmax=30, lmax=10000, tol=1e-10, precision=fg.FG_PREC_FP64)
    X16, st16 = fg.solve_batch(systems, Bs, Fs, kmax=30, lmax=10000, tol=1e-10, precision=fg.FG_PREC_MIXED16)
    for a, b, st in zip(X64, X16, st16):
        assert st["converged"] == 1 and st["true_rel_residual"] <= 1e-10
        assert np.linalg.norm(b[:-1] - a[:-1]) <= 1e-8 * np.linalg.norm(a[:-1])


def test_mixed16_needs_gram_path(fg):
    p = G.transport_problem(9)
    s = fg.transport_system(p)
    F = s.transport_assemble(p)
    with pytest.raises(Exception):
        fg.solve_batch([s], [F], [F], kmax=40, lmax=10, tol=1e-10, precision=fg.FG_PREC_MIXED16)
