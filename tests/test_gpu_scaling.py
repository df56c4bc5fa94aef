"""Diagonal scaling on the GPU (fg_scale, fg_unscale) against the CPU
restatement of Left_scaling_EBE / LeftRight_scaling_EBE / Left_unscaling
(oracle/ebe_gmres.c): scaled blocks and right-hand side bit-exact (the
accumulating Diag set-up is bit-exact, each entry is one product); the
scaled system solved without preconditioner and unscaled reaches the
solution of the unscaled system (rel-L2 1e-9 at tol 1e-10)."""
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


@pytest.mark.parametrize("kind", ["Left", "LeftRight"])
def test_scaling_bit_exact(fg, kind):
    p = G.transport_problem(33, angle_deg=25.0, k=1e-3)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    As, Fs, D, inv = O.scale(lm, A, m.neq, F, kind)
    s = fg.System(m)
    s.set_blocks(A)
    code = fg.FG_SCALE_LEFT if kind == "Left" else fg.FG_SCALE_LEFTRIGHT
    Fg = s.scale(code, F)
    assert np.array_equal(s.get_blocks(), As)
    assert np.array_equal(Fg[:-1], Fs[:-1])
    X = np.random.default_rng(2).standard_normal(m.neq + 1)
    X[-1] = 0
    assert np.array_equal(s.unscale(X)[:-1], O.unscale(inv, X)[:-1])


def test_leftright_scaled_solve(fg):
    p = G.transport_problem(65, angle_deg=30.0, k=1e-4)
    m = p.mesh
    A, F = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    X0, it0, *_ = O.ebe_diag_solve(lm, A, m.neq, F, perm, inv, kmax=30, lmax=1000, tol=1e-12)
    s = fg.System(m)
    s.set_blocks(A)
    Fs = s.scale(fg.FG_SCALE_LEFTRIGHT, F)
    r = s.solve(Fs, tol=1e-10)
    assert r.stats["converged"] == 1
    X = s.unscale(r.x)
    assert np.linalg.norm(X[:-1] - X0[:-1]) / np.linalg.norm(X0[:-1]) <= 1e-8


def test_block_scaling_bit_exact_and_solve(fg):
    """Block_scaling_EBE (Scaling "BlockScaling") on the device against the
    oracle (pinned to the reference's Block_scaling_EBE): scaled blocks and
    F bit-exact; the scaled system solves (no preconditioner) to the
    solution of the BlockDiag-preconditioned one, and fg_unscale is the
    identity."""
    p = G.obliquo_problem(17)
    m = p.mesh
    u = p.initial_state() * (1.0 + 0.02 * np.random.default_rng(3).standard_normal(m.neq))
    A, R = O.build_euler(p, u)
    bd, ibd, Id, Fo = O.blockdiag_setup(m, A, R, ref_quirks=True)
    As = O.block_scale(m, A, ibd)
    s = fg.euler_system(p)
    s.set_blocks(A)
    Fg = s.scale(fg.FG_SCALE_BLOCK, R)
    assert np.array_equal(s.get_blocks(), As.reshape(s.get_blocks().shape))
    assert np.array_equal(Fg[:-1], Fo[:-1])
    r = s.solve(Fg, tol=1e-12)
    assert r.stats["converged"] == 1
    assert np.array_equal(s.unscale(r.x)[:-1], r.x[:-1])
    s2 = fg.euler_system(p)
    s2.set_blocks(A)
    F2 = s2.precond_setup(fg.FG_PRECOND_BLOCKDIAG, fg.FG_SETUP_REF_QUIRKS, R)
    r2 = s2.solve(F2, tol=1e-12)
    assert np.linalg.norm(r.x[:-1] - r2.x[:-1]) <= 1e-8 * np.linalg.norm(r2.x[:-1])
